// Rigid fits: the FP64 Kabsch / Umeyama solution from the centred
// cross-covariance (SVD through the Jacobi eigen-decomposition of H^T H),
// shared by the RANSAC refit (device) and ICP (host, per iteration); and its
// FP32 three-point form for the RANSAC trials (jacobi3f / kabsch3f below).  Both users compile it without contraction (-fmad=false on the
// device, -ffp-contract=off on the host), so the two agree bit for bit.
#pragma once

#include <cmath>

namespace tdm {

__host__ __device__ inline void jacobi3(double A[3][3], double V[3][3], double ev[3]) {
  for (int i = 0; i < 3; ++i)
    for (int j = 0; j < 3; ++j) V[i][j] = (i == j) ? 1.0 : 0.0;
  for (int sweep = 0; sweep < 24; ++sweep) {
    double off = fabs(A[0][1]) + fabs(A[0][2]) + fabs(A[1][2]);
    double scale = fabs(A[0][0]) + fabs(A[1][1]) + fabs(A[2][2]);
    if (off <= 1e-300 || off <= 1e-18 * scale) break;
    for (int p = 0; p < 2; ++p)
      for (int q = p + 1; q < 3; ++q) {
        double apq = A[p][q];
        if (apq == 0.0) continue;
        double theta = (A[q][q] - A[p][p]) / (2.0 * apq);
        double t = 1.0 / (fabs(theta) + sqrt(theta * theta + 1.0));
        if (theta < 0.0) t = -t;
        double c = 1.0 / sqrt(t * t + 1.0), s = t * c;
        for (int k = 0; k < 3; ++k) {
          double akp = A[k][p], akq = A[k][q];
          A[k][p] = c * akp - s * akq;
          A[k][q] = s * akp + c * akq;
        }
        for (int k = 0; k < 3; ++k) {
          double apk = A[p][k], aqk = A[q][k];
          A[p][k] = c * apk - s * aqk;
          A[q][k] = s * apk + c * aqk;
        }
        for (int k = 0; k < 3; ++k) {
          double vkp = V[k][p], vkq = V[k][q];
          V[k][p] = c * vkp - s * vkq;
          V[k][q] = s * vkp + c * vkq;
        }
      }
  }
  for (int i = 0; i < 3; ++i) ev[i] = A[i][i];
}

// R (row-major) and t from the centred cross-covariance H = sum (y-cy)(x-cx)^T.
__host__ __device__ inline bool kabsch_from_h(const double H[3][3], const double cx[3], const double cy[3], double R[9],
                              double t[3]) {
  double M[3][3], V[3][3], ev[3];
  for (int i = 0; i < 3; ++i)
    for (int j = 0; j < 3; ++j) {
      double s = 0.0;
      for (int k = 0; k < 3; ++k) s += H[k][i] * H[k][j];
      M[i][j] = s;
    }
  jacobi3(M, V, ev);
  int o[3] = {0, 1, 2};
  for (int i = 0; i < 2; ++i)
    for (int j = 0; j < 2 - i; ++j)
      if (ev[o[j]] < ev[o[j + 1]]) { int tmp = o[j]; o[j] = o[j + 1]; o[j + 1] = tmp; }
  double v[3][3], u[3][3];
  for (int c = 0; c < 3; ++c)
    for (int r = 0; r < 3; ++r) v[c][r] = V[r][o[c]];
  v[2][0] = v[0][1] * v[1][2] - v[0][2] * v[1][1];
  v[2][1] = v[0][2] * v[1][0] - v[0][0] * v[1][2];
  v[2][2] = v[0][0] * v[1][1] - v[0][1] * v[1][0];
  for (int c = 0; c < 2; ++c) {
    double hv[3], n = 0.0;
    for (int r = 0; r < 3; ++r) {
      hv[r] = H[r][0] * v[c][0] + H[r][1] * v[c][1] + H[r][2] * v[c][2];
      n += hv[r] * hv[r];
    }
    n = sqrt(n);
    if (!(n > 1e-300)) return false;
    for (int r = 0; r < 3; ++r) u[c][r] = hv[r] / n;
  }
  {
    double d = u[0][0] * u[1][0] + u[0][1] * u[1][1] + u[0][2] * u[1][2], n = 0.0;
    for (int r = 0; r < 3; ++r) { u[1][r] = u[1][r] - d * u[0][r]; n += u[1][r] * u[1][r]; }
    n = sqrt(n);
    if (!(n > 1e-300)) return false;
    for (int r = 0; r < 3; ++r) u[1][r] = u[1][r] / n;
  }
  u[2][0] = u[0][1] * u[1][2] - u[0][2] * u[1][1];
  u[2][1] = u[0][2] * u[1][0] - u[0][0] * u[1][2];
  u[2][2] = u[0][0] * u[1][1] - u[0][1] * u[1][0];
  for (int i = 0; i < 3; ++i)
    for (int j = 0; j < 3; ++j) R[3 * i + j] = v[0][i] * u[0][j] + v[1][i] * u[1][j] + v[2][i] * u[2][j];
  for (int i = 0; i < 3; ++i) t[i] = cx[i] - (R[3 * i] * cy[0] + R[3 * i + 1] * cy[1] + R[3 * i + 2] * cy[2]);
  return true;
}

}  // namespace tdm

namespace tdm {

// RANSAC trial fit in FP32: the trial model is rounded to FP32 for the inlier
// tests anyway, and GB300 issues FP32 at many times its FP64 rate.  Same steps
// as jacobi3 / kabsch_from_h in single precision, with a sweep bound and a
// stopping rule sized for FP32 (off-diagonal below 1e-6 of the diagonal).
// Compiled without contraction on both sides, like the FP64 form.
__host__ __device__ inline void jacobi3f(float A[3][3], float V[3][3], float ev[3]) {
  for (int i = 0; i < 3; ++i)
    for (int j = 0; j < 3; ++j) V[i][j] = (i == j) ? 1.0f : 0.0f;
  for (int sweep = 0; sweep < 16; ++sweep) {
    const float off = fabsf(A[0][1]) + fabsf(A[0][2]) + fabsf(A[1][2]);
    const float scale = fabsf(A[0][0]) + fabsf(A[1][1]) + fabsf(A[2][2]);
    if (off <= 1e-30f || off <= 1e-6f * scale) break;
    for (int p = 0; p < 2; ++p)
      for (int q = p + 1; q < 3; ++q) {
        const float apq = A[p][q];
        if (apq == 0.0f) continue;
        const float theta = (A[q][q] - A[p][p]) / (2.0f * apq);
        float t = 1.0f / (fabsf(theta) + sqrtf(theta * theta + 1.0f));
        if (theta < 0.0f) t = -t;
        const float c = 1.0f / sqrtf(t * t + 1.0f), s = t * c;
        for (int k = 0; k < 3; ++k) {
          const float akp = A[k][p], akq = A[k][q];
          A[k][p] = c * akp - s * akq;
          A[k][q] = s * akp + c * akq;
        }
        for (int k = 0; k < 3; ++k) {
          const float apk = A[p][k], aqk = A[q][k];
          A[p][k] = c * apk - s * aqk;
          A[q][k] = s * apk + c * aqk;
        }
        for (int k = 0; k < 3; ++k) {
          const float vkp = V[k][p], vkq = V[k][q];
          V[k][p] = c * vkp - s * vkq;
          V[k][q] = s * vkp + c * vkq;
        }
      }
  }
  for (int i = 0; i < 3; ++i) ev[i] = A[i][i];
}

// x = R y + t from the three correspondences s[0..2] (R row-major), FP32.
// False when the fit is degenerate.
__host__ __device__ inline bool kabsch3f(const float* x, const float* y, const int s[3], float R[9], float t[3]) {
  float cx[3], cy[3];
  for (int a = 0; a < 3; ++a) {
    cx[a] = ((x[3 * s[0] + a] + x[3 * s[1] + a]) + x[3 * s[2] + a]) / 3.0f;
    cy[a] = ((y[3 * s[0] + a] + y[3 * s[1] + a]) + y[3 * s[2] + a]) / 3.0f;
  }
  float H[3][3] = {{0.0f, 0.0f, 0.0f}, {0.0f, 0.0f, 0.0f}, {0.0f, 0.0f, 0.0f}};
  for (int i = 0; i < 3; ++i) {
    float dx[3], dy[3];
    for (int a = 0; a < 3; ++a) { dx[a] = x[3 * s[i] + a] - cx[a]; dy[a] = y[3 * s[i] + a] - cy[a]; }
    for (int a = 0; a < 3; ++a)
      for (int b = 0; b < 3; ++b) H[a][b] += dy[a] * dx[b];
  }
  float M[3][3], V[3][3], ev[3];
  for (int i = 0; i < 3; ++i)
    for (int j = 0; j < 3; ++j) {
      float acc = 0.0f;
      for (int k = 0; k < 3; ++k) acc += H[k][i] * H[k][j];
      M[i][j] = acc;
    }
  jacobi3f(M, V, ev);
  int o[3] = {0, 1, 2};
  for (int i = 0; i < 2; ++i)
    for (int j = 0; j < 2 - i; ++j)
      if (ev[o[j]] < ev[o[j + 1]]) { int tmp = o[j]; o[j] = o[j + 1]; o[j + 1] = tmp; }
  float v[3][3], u[3][3];
  for (int c = 0; c < 3; ++c)
    for (int r = 0; r < 3; ++r) v[c][r] = V[r][o[c]];
  v[2][0] = v[0][1] * v[1][2] - v[0][2] * v[1][1];
  v[2][1] = v[0][2] * v[1][0] - v[0][0] * v[1][2];
  v[2][2] = v[0][0] * v[1][1] - v[0][1] * v[1][0];
  for (int c = 0; c < 2; ++c) {
    float hv[3], n = 0.0f;
    for (int r = 0; r < 3; ++r) {
      hv[r] = H[r][0] * v[c][0] + H[r][1] * v[c][1] + H[r][2] * v[c][2];
      n += hv[r] * hv[r];
    }
    n = sqrtf(n);
    if (!(n > 1e-30f)) return false;
    for (int r = 0; r < 3; ++r) u[c][r] = hv[r] / n;
  }
  {
    const float d = u[0][0] * u[1][0] + u[0][1] * u[1][1] + u[0][2] * u[1][2];
    float n = 0.0f;
    for (int r = 0; r < 3; ++r) { u[1][r] = u[1][r] - d * u[0][r]; n += u[1][r] * u[1][r]; }
    n = sqrtf(n);
    if (!(n > 1e-30f)) return false;
    for (int r = 0; r < 3; ++r) u[1][r] = u[1][r] / n;
  }
  u[2][0] = u[0][1] * u[1][2] - u[0][2] * u[1][1];
  u[2][1] = u[0][2] * u[1][0] - u[0][0] * u[1][2];
  u[2][2] = u[0][0] * u[1][1] - u[0][1] * u[1][0];
  for (int i = 0; i < 3; ++i)
    for (int j = 0; j < 3; ++j) R[3 * i + j] = v[0][i] * u[0][j] + v[1][i] * u[1][j] + v[2][i] * u[2][j];
  for (int i = 0; i < 3; ++i) t[i] = cx[i] - (R[3 * i] * cy[0] + R[3 * i + 1] * cy[1] + R[3 * i + 2] * cy[2]);
  return true;
}

}  // namespace tdm
