// Blackbody LUT of the renderer (src/blackbody.js): Planck spectra integrated against the analytic
// multi-lobe fit of the CIE 1931 observer at 2 nm, XYZ -> linear Rec.709 with a Bradford white balance to
// a blackbody at Twb, in doubles as the page computes it, stored as f32.
#include <algorithm>
#include <cmath>

#include "../../include/fire_sim.h"

namespace {

const double kH = 6.62607015e-34, kC = 2.99792458e8, kB = 1.380649e-23;

double lobe(double x, double mu, double s1, double s2) {   // src/blackbody.js:17
  const double t = (x - mu) / (x < mu ? s1 : s2);
  return std::exp(-0.5 * t * t);
}
void cie(double l, double out[3]) {   // src/blackbody.js:18-23
  out[0] = 1.056 * lobe(l, 599.8, 37.9, 31.0) + 0.362 * lobe(l, 442.0, 16.0, 26.7) - 0.065 * lobe(l, 501.1, 20.4, 26.2);
  out[1] = 0.821 * lobe(l, 568.8, 46.9, 40.5) + 0.286 * lobe(l, 530.9, 16.3, 31.1);
  out[2] = 1.217 * lobe(l, 437.0, 11.8, 36.0) + 0.681 * lobe(l, 459.0, 26.0, 13.8);
}
double planck(double lnm, double T) {   // src/blackbody.js:24-27
  const double l = lnm * 1e-9;
  return (2 * kH * kC * kC) / (std::pow(l, 5) * (std::exp((kH * kC) / (l * kB * T)) - 1));
}
// soot: spectral emissivity ~ lambda^-1.39 normalised at 550 nm (src/blackbody.js:29-37)
void blackbody_xyz(double T, bool soot, double out[3]) {
  double X = 0, Y = 0, Z = 0;
  for (int l = 380; l <= 780; l += 2) {
    const double p = planck(l, T) * (soot ? std::pow(l / 550.0, -1.39) : 1.0);
    double c[3];
    cie(l, c);
    X += p * c[0];
    Y += p * c[1];
    Z += p * c[2];
  }
  out[0] = X; out[1] = Y; out[2] = Z;
}
const double XYZ2RGB[3][3] = {{3.2404542, -1.5371385, -0.4985314}, {-0.9692660, 1.8760108, 0.0415560}, {0.0556434, -0.2040259, 1.0572252}};
const double XYZ2LMS[3][3] = {{0.8951, 0.2664, -0.1614}, {-0.7502, 1.7135, 0.0367}, {0.0389, -0.0685, 1.0296}};   // Bradford
const double D65[3] = {0.95047, 1.0, 1.08883};
void mul(const double M[3][3], const double v[3], double out[3]) {
  for (int r = 0; r < 3; ++r) out[r] = M[r][0] * v[0] + M[r][1] * v[1] + M[r][2] * v[2];
}
// inverse by cofactors, the page's formula (src/blackbody.js:50-60)
void inv3(const double m[3][3], double o[3][3]) {
  const double a = m[0][0], b = m[0][1], c2 = m[0][2], d = m[1][0], e = m[1][1], f = m[1][2], g2 = m[2][0], h2 = m[2][1], i = m[2][2];
  const double A = e * i - f * h2, B = -(d * i - f * g2), C = d * h2 - e * g2;
  const double det = a * A + b * B + c2 * C;
  o[0][0] = A / det; o[0][1] = -(b * i - c2 * h2) / det; o[0][2] = (b * f - c2 * e) / det;
  o[1][0] = B / det; o[1][1] = (a * i - c2 * g2) / det; o[1][2] = -(a * f - c2 * d) / det;
  o[2][0] = C / det; o[2][1] = -(a * h2 - b * g2) / det; o[2][2] = (a * e - b * d) / det;
}

}  // namespace

extern "C" int fire_blackbody_lut(int n, float tmin, float tmax, float twb, float* out) {
  if (!out || n < 2 || !(tmax > tmin)) return FIRE_ERR_BAD_ARG;
  double LMS2XYZ[3][3];
  inv3(XYZ2LMS, LMS2XYZ);
  double src[3] = {1, 1, 1}, dst[3] = {1, 1, 1};
  const bool wb = twb != 0.0f;
  if (wb) {   // whiteBalance (src/blackbody.js:65-75)
    double w[3];
    blackbody_xyz((double)twb, false, w);
    const double wn[3] = {w[0] / w[1], w[1] / w[1], w[2] / w[1]};
    mul(XYZ2LMS, wn, src);
    mul(XYZ2LMS, D65, dst);
  }
  double refv[3];
  blackbody_xyz(1500.0, false, refv);
  const double ref = refv[1];
  for (int row = 0; row < 2; ++row)
    for (int i = 0; i < n; ++i) {   // src/blackbody.js:79-92
      const double T = (double)tmin + ((double)tmax - (double)tmin) * i / (n - 1);
      double xyz[3];
      blackbody_xyz(T, row == 1, xyz);
      for (double& v : xyz) v /= ref;
      double rgb[3];
      if (wb) {
        double lms[3], x2[3];
        mul(XYZ2LMS, xyz, lms);
        for (int k = 0; k < 3; ++k) lms[k] = lms[k] * dst[k] / src[k];
        mul(LMS2XYZ, lms, x2);
        mul(XYZ2RGB, x2, rgb);
      } else {
        mul(XYZ2RGB, xyz, rgb);
      }
      float* o = out + 4 * ((size_t)row * n + i);
      o[0] = (float)std::max(0.0, rgb[0]);
      o[1] = (float)std::max(0.0, rgb[1]);
      o[2] = (float)std::max(0.0, rgb[2]);
      o[3] = (float)xyz[1];
    }
  return FIRE_OK;
}
