// The photon-map handle (skw_photon_map), shared by the host translation
// units that build it (skw_photon_map.cpp) and render with it
// (skw_render_api.cpp).
#pragma once

#include <cstdint>
#include <limits>
#include <vector>

#include "photon_types.h"
#include "skw_internal.h"

namespace skw {

// One photon kd-tree on the device: KdNode per tree position plus the
// photon's normal id, incident-direction id and weight in tree order.
struct PhotonMapData {
  int64_t n = 0;
  int64_t paths = 0;
  std::vector<PhotonRec> input;  // the photons in the order they were given (path order)
  std::vector<int32_t> perm;     // tree position -> input index
  void *d_nodes = nullptr;
  uint16_t *d_nids = nullptr, *d_dirid = nullptr;
  float *d_weight = nullptr;
  bool built_on_gpu = false;     // the tree came from the GPU builder
};

}  // namespace skw

struct skw_photon_map {
  skw_ctx *ctx = nullptr;
  skw::PhotonMapData maps[3];  // caustic, direct, indirect
  double scene_area = 0.0;
  double lookup_dist[3] = {0, 0, 0};  // irradiance-estimate radii per map
  // irradiance photons, tree order
  int64_t n_irr = 0;
  std::vector<float> irr_pos, irr_ext, irr_int;
  std::vector<uint16_t> irr_nrm;
  void *d_irr_nodes = nullptr;
  uint16_t *d_irr_nids = nullptr;
  float *d_irr_ext = nullptr, *d_irr_int = nullptr;
  double max_irr_dist = std::numeric_limits<double>::infinity();
  double *d_dirs = nullptr;
  unsigned *d_status = nullptr;
  double shoot_ms = 0.0, build_ms = 0.0;
};

