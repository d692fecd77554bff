// Host restatement of the reference's measured BRDF
// (Raytracer/BxDFs/MERLMeasured.cpp:24-423): the loader (scaling, colour
// conversion to spectrum coefficients, half precision), the sampling
// segmentations (_InitializeSegmentations, Segmentation2D, _Reduce) and the
// evaluation, sampling and density in double.  Compiled with
// -ffp-contract=off; the arithmetic follows the reference operation by
// operation so that the tables are bit-identical.
#include "merl.h"

#include <algorithm>
#include <cmath>
#include <cstring>
#include <limits>

namespace skw {
namespace {

constexpr double kPi = 3.14159265358979323846, kPi2 = 1.57079632679489661923, kInvPi = 0.31830988618379067154;

// The loader's colour conversion (Core/Color.cpp global_sRGB_E_ColorSystem
// RGB_To_XYZ, then SpectrumRoutines::XYZToSpectrumCoef): two 3x3 matrices,
// each row applied as (m0 v0 + m1 v1) + m2 v2.
const double kRgbToXyz[3][3] = {{0x1.fcd8dcf9c3460p-2, 0x1.5b3a5407f3635p-2, 0x1.4fd99dfc92adap-3},
                                {0x1.065fd1f0c8b0dp-2, 0x1.5b3a5407f3631p-1, 0x1.0cae17fd42268p-4},
                                {0x1.7da2a5bb5271ep-6, 0x1.cef8700a99da9p-4, 0x1.ba33dcd0d2310p-1}};
const double kXyzToCoef[3][3] = {{0x1.368e683d1c8e4p-4, -0x1.0c40314b9028fp-3, 0x1.0e07e946862fdp+0},
                                 {-0x1.432fb70f599bep+0, 0x1.14a5623a99345p+1, 0x1.9e954c8d546b1p-4},
                                 {0x1.040236acfe51bp+1, -0x1.6cd6c8f911e96p-1, -0x1.4672dbc94b232p-2}};
// Row Y of the spectrum-to-XYZ matrix (luminance weights).
const double kLum[3] = {0x1.b38293da589a6p-5, 0x1.2b993cc221566p-1, 0x1.725d3400723f6p-2};

void mat3(const double m[3][3], const double v[3], double o[3]) {
  for (int i = 0; i < 3; ++i) o[i] = (m[i][0] * v[0] + m[i][1] * v[1]) + m[i][2] * v[2];
}

double luminance(const double s[3]) {
  double r = 0.0;
  for (int j = 0; j < 3; ++j) r += kLum[j] * s[j];
  return r;
}

// IEEE binary16 from float, round to nearest even (the half class of
// Math/Half, OpenEXR's conversion).
uint16_t float_to_half(float f) {
  uint32_t x;
  std::memcpy(&x, &f, 4);
  const uint32_t sign = (x >> 16) & 0x8000u;
  const int32_t e = (int32_t)((x >> 23) & 0xFF) - 127 + 15;
  uint32_t m = x & 0x7FFFFFu;
  if (((x >> 23) & 0xFF) == 0xFF) return (uint16_t)(sign | 0x7C00u | (m ? 0x200u : 0));  // inf / nan
  if (e <= 0) {
    if (e < -10) return (uint16_t)sign;  // underflow to zero
    m |= 0x800000u;
    const int s = 14 - e;
    const uint32_t a = (1u << (s - 1)) - 1, b = (m >> s) & 1u;
    return (uint16_t)(sign | ((m + a + b) >> s));
  }
  m = m + 0xFFFu + ((m >> 13) & 1u);
  uint32_t ee = (uint32_t)e;
  if (m & 0x800000u) {
    m = 0;
    ee += 1;
  }
  if (ee > 30) return (uint16_t)(sign | 0x7C00u);  // overflow to infinity
  return (uint16_t)(sign | (ee << 10) | (m >> 13));
}

double half_to_double(uint16_t h) {
  const uint32_t sign = (h & 0x8000u) << 16, e = (h >> 10) & 0x1F, m = h & 0x3FFu;
  uint32_t x;
  if (e == 0) {
    if (m == 0) {
      x = sign;
    } else {  // subnormal
      int k = 0;
      uint32_t mm = m;
      while (!(mm & 0x400u)) {
        mm <<= 1;
        ++k;
      }
      x = sign | ((uint32_t)(127 - 15 + 1 - k) << 23) | ((mm & 0x3FFu) << 13);
    }
  } else if (e == 31) {
    x = sign | 0x7F800000u | (m << 13);
  } else {
    x = sign | ((e - 15 + 127) << 23) | (m << 13);
  }
  float f;
  std::memcpy(&f, &x, 4);
  return (double)f;
}

void spherical_direction(double phi, double theta, double v[3]) {
  const double st = std::sin(theta), ct = std::cos(theta);
  v[0] = st * std::cos(phi);
  v[1] = st * std::sin(phi);
  v[2] = ct;
}

double spherical_theta(const double v[3]) { return std::acos(std::min(1.0, std::max(-1.0, v[2]))); }

double spherical_phi(const double v[3]) {
  const double p = std::atan2(v[1], v[0]);
  return p < 0.0 ? p + 2.0 * kPi : p;
}

double dot3(const double a[3], const double b[3]) { return a[0] * b[0] + a[1] * b[1] + a[2] * b[2]; }

// MERLMeasuredData::GetBRDF (MERLMeasured.cpp:254-293).
void get_brdf(const std::vector<uint16_t> &t, const double wi[3], const double wo[3], double f[3]) {
  double h[3] = {wi[0] + wo[0], wi[1] + wo[1], wi[2] + wo[2]};
  f[0] = f[1] = f[2] = 0.0;
  if (h[0] == 0.0 && h[1] == 0.0 && h[2] == 0.0) return;
  const double ls = h[0] * h[0] + h[1] * h[1] + h[2] * h[2];
  if (ls > 0.0) {
    const double inv = 1.0 / std::sqrt(ls);
    for (double &c : h) c = c * inv;
  }
  // MathRoutines::SphericalAngles (Math/MathRoutines.h:394-411)
  const double sin_t = std::sqrt(h[0] * h[0] + h[1] * h[1]), cos_t = h[2];
  double sin_p = 0.0, cos_p = 1.0;
  if (sin_t > 1e-10) {
    const double inv = 1.0 / sin_t;
    sin_p = h[1] * inv;
    cos_p = h[0] * inv;
  }
  const double whx[3] = {cos_p * cos_t, sin_p * cos_t, -sin_t}, why[3] = {-sin_p, cos_p, 0.0};
  const double diff[3] = {dot3(wi, whx), dot3(wi, why), dot3(wi, h)};
  const double th = spherical_theta(h), td = spherical_theta(diff), pd = spherical_phi(diff);
  const size_t ipd = (size_t)(pd * kInvPi * kMerlPhiD) % kMerlPhiD;
  const size_t itd = std::min((size_t)(td * 2.0 * kInvPi * kMerlThetaD), (size_t)kMerlThetaD - 1);
  const double ths = std::sqrt(th * 2.0 * kInvPi) * kMerlThetaH;
  const size_t ith = std::min((size_t)ths, (size_t)kMerlThetaH - 1);
  const size_t idx = ipd + (itd + ith * kMerlThetaD) * kMerlPhiD;
  if (idx < (size_t)(kMerlThetaH - 1) * kMerlThetaD * kMerlPhiD) {
    const double w = ths - (size_t)ths;
    const size_t j = idx + (size_t)kMerlThetaD * kMerlPhiD;
    for (int c = 0; c < 3; ++c) f[c] = half_to_double(t[3 * idx + c]) * (1.0 - w) + half_to_double(t[3 * j + c]) * w;
  } else {
    for (int c = 0; c < 3; ++c) f[c] = half_to_double(t[3 * idx + c]);
  }
}

// Segmentation2D::_Reduce (MERLMeasured.cpp:90-118).
std::vector<size_t> reduce(std::vector<float> v, size_t size) {
  const int iterations = (int)v.size() - (int)size;
  std::vector<size_t> ret(v.size());
  for (size_t i = 0; i < v.size(); ++i) ret[i] = i;
  for (int it = 0; it < iterations; ++it) {
    float best = std::numeric_limits<float>::infinity();
    size_t ind = 0;
    for (size_t j = 0; j + 1 < ret.size(); ++j) {
      const float tmp = v[j] + v[j + 1];
      if (tmp < best) {
        best = tmp;
        ind = j;
      }
    }
    v[ind] += v[ind + 1];
    v.erase(v.begin() + ind + 1);
    ret.erase(ret.begin() + ind + 1);
  }
  return ret;
}

// Segmentation2D(values) (MERLMeasured.cpp:24-84) into its kSegFloats slot.
void segmentation(const std::vector<std::vector<float>> &values, float *out) {
  const size_t sx = kSegPhi, sy = kSegTheta, n = values.size(), m = values[0].size();
  std::vector<float> sum_x(m, 0.f), sum_y(n, 0.f);
  for (size_t i = 0; i < n; ++i)
    for (size_t j = 0; j < m; ++j) {
      sum_x[j] += values[i][j];
      sum_y[i] += values[i][j];
    }
  const std::vector<size_t> rx = reduce(sum_x, sx), ry = reduce(sum_y, sy);
  float *cols = out, *rows = out + sy * sx, *gx = rows + sy, *gy = gx + sx;
  for (size_t i = 0; i < sx; ++i) gx[i] = rx[i] / (float)m;
  for (size_t i = 0; i < sy; ++i) gy[i] = ry[i] / (float)n;
  for (size_t i = 0; i < sy; ++i)
    for (size_t j = 0; j < sx; ++j) {
      float &c = cols[i * sx + j];
      c = j > 0 ? cols[i * sx + j - 1] : 0.f;
      const size_t ey = i + 1 < sy ? ry[i + 1] : n, ex = j + 1 < sx ? rx[j + 1] : m;
      for (size_t i1 = ry[i]; i1 < ey; ++i1)
        for (size_t j1 = rx[j]; j1 < ex; ++j1) c += values[i1][j1];
    }
  for (size_t i = 0; i < sy; ++i) {
    rows[i] = i > 0 ? rows[i - 1] : 0.f;
    rows[i] += cols[i * sx + sx - 1];
  }
  for (size_t i = 0; i < sy; ++i) {
    rows[i] /= rows[sy - 1];
    const double inv = 1.0 / cols[i * sx + sx - 1];
    for (size_t j = 0; j < sx; ++j) cols[i * sx + j] = (float)(cols[i * sx + j] * inv);
  }
}

// MathRoutines::BinarySearchCDF over floats (Math/MathRoutines.h:191-218).
size_t search_cdf(const float *cdf, size_t n, double u, double *pdf) {
  size_t b = 0, e = n - 1;
  while (b < e) {
    const size_t mid = b + (e - b) / 2;
    if (cdf[mid] <= u) b = mid + 1; else e = mid;
  }
  *pdf = b == 0 ? cdf[0] : (double)(cdf[b] - cdf[b - 1]);  // the difference of two floats, in float
  return b;
}

size_t incident_bin(const double wi[3]) {
  return std::min((size_t)(spherical_theta(wi) * 2.0 * kInvPi * kSegIncident), (size_t)kSegIncident - 1);
}

// MERLMeasuredData::PDF (:342-369).
double data_pdf(const MerlHost &m, const double wi[3], const double wo[3]) {
  const float *seg = m.seg.data() + incident_bin(wi) * kSegFloats;
  const float *cols = seg, *rows = seg + kSegTheta * kSegPhi, *gx = rows + kSegTheta, *gy = gx + kSegPhi;
  const double ip = spherical_phi(wi), ep = spherical_phi(wo), et = spherical_theta(wo);
  double dp = std::fabs(ip - ep);
  if (dp > kPi) dp = 2.0 * kPi - dp;
  const double px = dp * kInvPi, py = et * 2.0 * kInvPi;
  // Segmentation2D::PDF (:148-169): upper_bound over the grid lines
  size_t ci = (size_t)(std::upper_bound(gx, gx + kSegPhi, px) - gx), ri = (size_t)(std::upper_bound(gy, gy + kSegTheta, py) - gy);
  --ci;
  --ri;
  const double bx0 = gx[ci], by0 = gy[ri];
  const double bx1 = ci + 1 < (size_t)kSegPhi ? gx[ci + 1] : 1.0, by1 = ri + 1 < (size_t)kSegTheta ? gy[ri + 1] : 1.0;
  const float *cc = cols + ri * kSegPhi;
  const double row_pdf = ri > 0 ? (double)(rows[ri] - rows[ri - 1]) : rows[ri];
  const double col_pdf = ci > 0 ? (double)(cc[ci] - cc[ci - 1]) : cc[ci];
  const double pdf = row_pdf * col_pdf;
  const double d_phi = (bx1 - bx0) * kPi;
  const double d_cos = std::cos(by0 * kPi2) - std::cos(by1 * kPi2);
  return 0.5 * pdf / (d_phi * d_cos);
}

}  // namespace

bool merl_load(const void *bytes, int64_t n_bytes, MerlHost &out) {
  if (!bytes || n_bytes < 12) return false;
  int32_t dims[3];
  std::memcpy(dims, bytes, 12);
  if ((int64_t)dims[0] * dims[1] * dims[2] != kMerlN) return false;
  if (n_bytes < 12 + (int64_t)3 * kMerlN * 8) return false;
  const char *p = (const char *)bytes + 12;
  const double scales[3] = {1.0 / 1500, 1.15 / 1500, 1.66 / 1500};
  out.table.assign((size_t)3 * kMerlN, 0);
  for (int i = 0; i < kMerlN; ++i) {
    double rgb[3], xyz[3], coef[3];
    for (int c = 0; c < 3; ++c) {
      double v;
      std::memcpy(&v, p + ((size_t)c * kMerlN + i) * 8, 8);
      rgb[c] = std::max(0.0, v * scales[c]);
    }
    mat3(kRgbToXyz, rgb, xyz);
    mat3(kXyzToCoef, xyz, coef);
    for (int c = 0; c < 3; ++c) out.table[(size_t)3 * i + c] = float_to_half((float)coef[c]);
  }
  // _InitializeSegmentations (:219-251)
  const size_t etr = (size_t)kSegMul * kSegTheta, epr = (size_t)kSegMul * kSegPhi;
  const double phi_coef = kPi / epr, theta_coef = kPi2 / etr;
  out.seg.assign((size_t)kSegIncident * kSegFloats, 0.f);
  std::vector<std::vector<float>> values(etr, std::vector<float>(epr));
  for (int i = 0; i < kSegIncident; ++i) {
    double inc[3];
    spherical_direction(0.0, (i + 0.5) * kPi2 / kSegIncident, inc);
    for (size_t i1 = 0; i1 < etr; ++i1) {
      const double et = (i1 + 0.5) * theta_coef, cos_et = std::cos(et);
      const double d_cos = std::cos(i1 * theta_coef) - std::cos((i1 + 1) * theta_coef);
      for (size_t j1 = 0; j1 < epr; ++j1) {
        double ex[3], f[3];
        spherical_direction((j1 + 0.5) * phi_coef, et, ex);
        get_brdf(out.table, inc, ex, f);
        values[i1][j1] = (float)(phi_coef * d_cos * cos_et * luminance(f));
      }
    }
    segmentation(values, out.seg.data() + (size_t)i * kSegFloats);
  }
  return true;
}

void merl_eval(const MerlHost &m, const double wi[3], const double wo[3], double f[3], double *pdf) {
  // MERLMeasured::Evaluate / PDF (:378-423): the incident side's hemisphere is folded to +z
  f[0] = f[1] = f[2] = 0.0;
  *pdf = 0.0;
  if (wi[2] * wo[2] < 0.0) return;
  double a[3] = {wi[0], wi[1], wi[2]}, b[3] = {wo[0], wo[1], wo[2]};
  if (wi[2] < 0.0) {
    a[2] = -a[2];
    b[2] = -b[2];
  }
  get_brdf(m.table, a, b, f);
  *pdf = data_pdf(m, a, b);
}

void merl_sample(const MerlHost &m, const double wi[3], const double u[2], double wo[3], double f[3], double *pdf) {
  // MERLMeasured::Sample (:397-411) + MERLMeasuredData::Sample (:296-340)
  const bool flip = wi[2] < 0.0;
  const double a[3] = {wi[0], wi[1], flip ? -wi[2] : wi[2]};
  const float *seg = m.seg.data() + incident_bin(a) * kSegFloats;
  const float *cols = seg, *rows = seg + kSegTheta * kSegPhi, *gx = rows + kSegTheta, *gy = gx + kSegPhi;
  double s0 = u[0], s1 = u[1];
  bool opposite = false;
  if (s0 > 0.5) {
    opposite = true;
    s0 = (s0 - 0.5) * 2.0;
  } else {
    s0 *= 2.0;
  }
  double row_pdf, col_pdf;
  const size_t ri = search_cdf(rows, kSegTheta, s1, &row_pdf);
  const float *cc = cols + ri * kSegPhi;
  const size_t ci = search_cdf(cc, kSegPhi, s0, &col_pdf);
  const double r0 = (s0 - (ci > 0 ? cc[ci - 1] : 0.0)) / col_pdf;
  const double r1 = (s1 - (ri > 0 ? rows[ri - 1] : 0.0)) / row_pdf;
  const double bx0 = gx[ci], by0 = gy[ri];
  const double bx1 = ci + 1 < (size_t)kSegPhi ? gx[ci + 1] : 1.0, by1 = ri + 1 < (size_t)kSegTheta ? gy[ri + 1] : 1.0;
  const double p = row_pdf * col_pdf;
  const double d_phi = (bx1 - bx0) * kPi;
  const double c1 = std::cos(by0 * kPi2), c2 = std::cos(by1 * kPi2), d_cos = c1 - c2;
  double phi = (bx0 + (bx1 - bx0) * r0) * kPi;
  if (opposite) phi = 2.0 * kPi - phi;
  phi += spherical_phi(a);
  const double ct = c1 - r1 * d_cos, st = std::sqrt(1.0 - ct * ct);
  wo[0] = st * std::cos(phi);
  wo[1] = st * std::sin(phi);
  wo[2] = ct;
  *pdf = 0.5 * p / (d_phi * d_cos);
  get_brdf(m.table, a, wo, f);
  if (flip) wo[2] = -wo[2];
}

}  // namespace skw
