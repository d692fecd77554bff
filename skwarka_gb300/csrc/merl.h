// Measured BRDF in the MERL layout (BxDFs/MERLMeasured.{h,cpp}): host-side
// table, sampling segmentations and the reference's evaluation, plus the
// device view used by the shading kernels.
#pragma once

#include <cstdint>
#include <vector>

namespace skw {

constexpr int kMerlThetaH = 90, kMerlThetaD = 90, kMerlPhiD = 180;  // MERLMeasured.h:75-77
constexpr int kMerlN = kMerlThetaH * kMerlThetaD * kMerlPhiD;
constexpr int kSegIncident = 90, kSegTheta = 24, kSegPhi = 45, kSegMul = 8;  // :81-87
// Floats per incident-theta segmentation: column CDFs, row CDF, X and Y grid lines.
constexpr int kSegFloats = kSegTheta * kSegPhi + kSegTheta + kSegPhi + kSegTheta;

// Device view of one measured BRDF.
struct MerlDev {
  const uint16_t *table;  // half RGB per entry (the loader's converted values)
  const float *seg;       // kSegIncident * kSegFloats
};

struct MerlHost {
  std::vector<uint16_t> table;  // 3 * kMerlN halves
  std::vector<float> seg;       // kSegIncident * kSegFloats
};

// MERLMeasuredData(std::istream&) on a file image: false if malformed.
bool merl_load(const void *bytes, int64_t n_bytes, MerlHost &out);
// GetBRDF / MERLMeasured::{Evaluate, PDF, Sample} in double, as the reference.
void merl_eval(const MerlHost &m, const double wi[3], const double wo[3], double f[3], double *pdf);
void merl_sample(const MerlHost &m, const double wi[3], const double u[2], double wo[3], double f[3], double *pdf);

}  // namespace skw
