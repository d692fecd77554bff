// Photon-map data shared by the host layer (skw_photon_map.cpp) and the
// kernels (photon.cu).
#pragma once

#include <cstdint>

namespace skw {

// A deposited photon (PhotonLTEIntegrator::Photon,
// LTEIntegrators/PhotonLTEIntegrator/PhotonInternalTypes.h:35-59): position,
// weight and the 16-bit CompressedDirection ids of the incident direction and
// of the surface's geometric normal.  28 bytes, the layout of skw_photon.
struct PhotonRec {
  float p[3];
  float w[3];
  uint16_t dir, nrm;
};
static_assert(sizeof(PhotonRec) == 28, "skw_photon layout");

// Photon emission: one entry per light in the reference's order (delta
// lights, then area lights), with the normalised cumulative luminance of
// the lights' power (PhotonLTEIntegrator::_GetLightsPowerCDF,
// PhotonLTEIntegrator.cpp:80-125).
struct PhotonLight {
  double cdf;
  int32_t kind;   // 0 point light, 1 area light
  int32_t index;  // into SceneDev::point_lights / area_lights
};

struct PhotonShootArgs {
  const PhotonLight *lights;
  int32_t n_lights;
  int32_t max_bounces;      // intersections per path
  float rr_probability;     // > 0: fixed Russian-roulette continue probability; 0: the reference's luminance rule
  uint64_t seed;
  // Indirect-photon slots per path in a chunk's staging (<= max_bounces - 1);
  // a path that would deposit more raises *overflow and the chunk is shot
  // again with every slot (its photons then depend on nothing but the path).
  int32_t slots;
  int *overflow;
};

}  // namespace skw

namespace skw {

// What the final-gather stages read: the indirect photon map (tree order) and
// the irradiance photon map (tree order), plus the direction table.
// The caustic map of a render (_LookupCausticRadiance,
// PhotonLTEIntegrator.cpp:579-627): its tree, photons in tree order, number
// of paths, and the lookup's k and radius.
struct CausticMap {
  const void *nodes;
  const uint16_t *nids;
  const uint16_t *dirid;
  const float *weight;
  int32_t n;
  double paths;
  int32_t k;
  double max_dist;
  const double *dirs;
};

struct GatherMaps {
  const void *ind_nodes;
  const uint16_t *ind_nids;
  const uint16_t *ind_dirid;
  int32_t n_ind;
  double ind_lookup_dist;  // sqrt(area / n_indirect * 32 / pi)
  const void *irr_nodes;
  const uint16_t *irr_nids;
  const float *irr_ext, *irr_int;
  int32_t n_irr;
  double max_irr_dist;
  const double *dirs;
  float lo[3], hi[3];  // the scene's bounds (the gather hits' spatial bins)
};

}  // namespace skw
