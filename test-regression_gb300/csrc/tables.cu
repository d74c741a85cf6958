// Per-condition-set tables of the mixed-precision and warm-start forms
// (host code).
//
// With an amplitude-independent covariance C = pederr^2 * R, every channel of
// a condition set shares L = pederr * L_R with L_R = chol(R), so the
// whitened problem of a channel is
//     min || G x - y ||^2,   G = L_R^-1 P (shared),  y = L_R^-1 s (per channel)
// scaled by 1/pederr^2 (the solution does not depend on pederr). The least-
// squares solution restricted to a passive set S is x_S = G_S^+ y with the
// pseudo-inverse G_S^+ = (G_S^T G_S)^-1 G_S^T, which depends on S only. The
// engine therefore builds, once per condition set, the pseudo-inverse of
// every non-empty S (columns in ascending order) by Householder QR in long
// double, and stores it in FP64, FP32 and as a float pair (hi + lo, for the
// double-float judge; p x N rows per set, packed). A
// passive-set solve on the device is then one small matrix-vector product read
// from an L1/L2-resident table;
// its error is ~cond(G_S) * eps (the QR-level bound), not cond(G_S)^2 * eps
// as for normal equations -- which matters here, since cond(G) reaches 5e4
// for the ECAL pulse and FP32 normal equations would break down.
#include <cmath>
#include <cstring>
#include <vector>

#include "mf_internal.h"

namespace mfgb {

namespace {

typedef long double ld;

// Householder QR of the N x p matrix A (column-major, ld N); returns R (p x p
// upper, row-major) and the p x N operator R^-1 Q^T (row-major), i.e. A^+.
bool pinv_qr(const ld* A, int N, int p, ld* pinv) {
  std::vector<ld> Q(A, A + N * p);  // overwritten by the Householder vectors
  std::vector<ld> R(p * p, 0), beta(p, 0);
  for (int k = 0; k < p; ++k) {
    ld norm = 0;
    for (int i = k; i < N; ++i) norm += Q[k * N + i] * Q[k * N + i];
    norm = std::sqrt(norm);
    if (norm == 0) return false;
    const ld alpha = Q[k * N + k] > 0 ? -norm : norm;
    Q[k * N + k] -= alpha;  // v = a - alpha e_k
    ld vnorm2 = 0;
    for (int i = k; i < N; ++i) vnorm2 += Q[k * N + i] * Q[k * N + i];
    beta[k] = vnorm2 > 0 ? 2 / vnorm2 : 0;
    for (int j = k + 1; j < p; ++j) {
      ld d = 0;
      for (int i = k; i < N; ++i) d += Q[k * N + i] * Q[j * N + i];
      d *= beta[k];
      for (int i = k; i < N; ++i) Q[j * N + i] -= d * Q[k * N + i];
    }
    R[k * p + k] = alpha;
    for (int j = k + 1; j < p; ++j) R[k * p + j] = Q[j * N + k];
  }
  // columns of Q^T applied to unit vectors: pinv = R^-1 (Q^T) restricted to p rows
  std::vector<ld> QT(p * N, 0);  // rows 0..p-1 of Q^T = H_{p-1} ... H_0 applied to e_i
  for (int i = 0; i < N; ++i) {
    std::vector<ld> e(N, 0);
    e[i] = 1;
    for (int k = 0; k < p; ++k) {
      ld d = 0;
      for (int r = k; r < N; ++r) d += Q[k * N + r] * e[r];
      d *= beta[k];
      for (int r = k; r < N; ++r) e[r] -= d * Q[k * N + r];
    }
    for (int r = 0; r < p; ++r) QT[r * N + i] = e[r];
  }
  for (int i = 0; i < N; ++i) {
    for (int r = p - 1; r >= 0; --r) {
      ld t = QT[r * N + i];
      for (int c = r + 1; c < p; ++c) t -= R[r * p + c] * pinv[c * N + i];
      pinv[r * N + i] = t / R[r * p + r];
    }
  }
  return true;
}

}  // namespace

int build_mixed_tables(const DevConditions& c, HostTables* t) {
  const int N = c.N, K = c.K;
  // L_R = chol(R) and W = L_R^-1 in long double
  ld L[KMAX][KMAX] = {}, W[KMAX][KMAX] = {};
  for (int i = 0; i < N; ++i)
    for (int j = 0; j <= i; ++j) {
      ld s = c.R[j * N + i];
      for (int k = 0; k < j; ++k) s -= L[i][k] * L[j][k];
      if (i == j) {
        if (!(s > 0)) return MF_EINVAL;  // samplecor not positive definite
        L[i][i] = std::sqrt(s);
      } else {
        L[i][j] = s / L[j][j];
      }
    }
  for (int col = 0; col < N; ++col)
    for (int i = 0; i < N; ++i) {
      ld s = (i == col) ? 1 : 0;
      for (int k = col; k < i; ++k) s -= L[i][k] * W[k][col];
      W[i][col] = i < col ? 0 : s / L[i][i];
    }
  ld G[KMAX * KMAX];
  for (int k = 0; k < K; ++k)
    for (int i = 0; i < N; ++i) {
      ld s = 0;
      for (int j = 0; j <= i; ++j) s += W[i][j] * ld(c.P[k * N + j]);
      G[k * N + i] = s;
    }
  t->N = N;
  t->K = K;
  int w = 0;
  for (int i = 0; i < N; ++i)
    for (int j = 0; j <= i; ++j, ++w) {
      t->W64[w] = double(W[i][j]);
      t->W32[w] = float(W[i][j]);
      t->W32lo[w] = float(W[i][j] - ld(t->W32[w]));
    }
  for (int e = 0; e < N * K; ++e) {
    t->G64[e] = double(G[e]);
    t->G32[e] = float(G[e]);
    t->G32lo[e] = float(G[e] - ld(t->G32[e]));
    t->P32[e] = float(c.P[e]);
    t->P32lo[e] = float(c.P[e] - double(t->P32[e]));
  }
  for (int i = 0; i < K; ++i) {
    ld nrm = 0;
    for (int j = 0; j < K; ++j) {
      ld s = 0;
      for (int r = 0; r < N; ++r) s += G[i * N + r] * G[j * N + r];
      t->H64[i * KMAX + j] = double(s);
      t->H32[i * KMAX + j] = float(s);
      if (i == j) nrm = s;
    }
    t->gnorm2[i] = double(nrm);
  }
  for (int k = 0; k < K; ++k) {
    int fz = N;
    for (int i = 0; i < N; ++i)
      if (G[k * N + i] != 0) { fz = i; break; }
    t->gfz[k] = fz;
  }
  // pseudo-inverses of every non-empty passive set: the p rows of the set's
  // columns (ascending), p x N row-major, packed back to back
  const int nmask = 1 << K;
  t->offset.assign(nmask + 1, 0);
  int total = 0;
  for (int m = 0; m < nmask; ++m) {
    t->offset[m] = total;
    total += __builtin_popcount(unsigned(m)) * N;
  }
  t->offset[nmask] = total;  // followed by one zero row (the branch-free solves read it)
  t->pinv64.assign(total + N, 0.0);
  t->pinv32.assign(total + N, 0.0f);
  t->pinv32lo.assign(total + N, 0.0f);
  std::vector<ld> A(N * KMAX), pinv(KMAX * N);
  for (int m = 1; m < nmask; ++m) {
    int p = 0;
    for (int k = 0; k < K; ++k)
      if (m & (1 << k)) {
        for (int i = 0; i < N; ++i) A[p * N + i] = G[k * N + i];
        ++p;
      }
    if (!pinv_qr(A.data(), N, p, pinv.data())) return MF_EINVAL;  // a zero pulse column
    for (int e = 0; e < p * N; ++e) {
      t->pinv64[t->offset[m] + e] = double(pinv[e]);
      t->pinv32[t->offset[m] + e] = float(pinv[e]);
      t->pinv32lo[t->offset[m] + e] = float(pinv[e] - ld(t->pinv32[t->offset[m] + e]));
    }
  }
  // the same operators as (hi, lo) pairs, for the double-float solve: with N
  // even every row (offset[m] + r N elements, 8 bytes each) starts on a
  // 16-byte boundary, so a row is N / 2 16-byte loads
  // followed by G as pairs, column by column (the double-float judge reads a
  // column per loop step, the same address in every lane)
  t->g2_off = 2 * (total + N);
  t->pinv2.assign(size_t(t->g2_off) + 2 * size_t(K) * N, 0.0f);
  for (int e = 0; e < total + N; ++e) {
    t->pinv2[2 * size_t(e)] = t->pinv32[e];
    t->pinv2[2 * size_t(e) + 1] = t->pinv32lo[e];
  }
  for (int e = 0; e < K * N; ++e) {
    t->pinv2[size_t(t->g2_off) + 2 * size_t(e)] = t->G32[e];
    t->pinv2[size_t(t->g2_off) + 2 * size_t(e) + 1] = t->G32lo[e];
  }
  return MF_OK;
}

}  // namespace mfgb
