// anderson.cuh -- the coefficient solve of the Anderson-accelerated
// PageRank solves (one vector in pagerank.cu, one per column in
// ppr_batch.cu).
//
// With q_j = r_{k-j} the residuals of the last three sweeps (newest first)
// and G their Gram matrix (G[i][j] = q_i . q_j), minimise
// || q_0 - g1 (q_0 - q_1) - g2 (q_1 - q_2) ||_2 over the m differences
// available (normal equations from G); the next input is then
// x_{k+1} = (1 - g1) g_k + (g1 - g2) g_{k-1} + g2 g_{k-2}.  Ill-conditioned
// systems or large coefficients fall back to fewer differences, down to the
// plain step x_{k+1} = g_k.
#pragma once

namespace tbsla {

// coef[0..2]: the weights of g_k, g_{k-1}, g_{k-2} (summing to 1); returns
// the number of older outputs in use (0, 1 or 2)
__device__ __forceinline__ int aa_coefficients(const double (&G)[3][3], int m, double (&coef)[3]) {
  double g1 = 0, g2 = 0;
  if (m == 2) {
    const double a11 = G[0][0] - 2 * G[0][1] + G[1][1];
    const double a12 = G[0][1] - G[0][2] - G[1][1] + G[1][2];
    const double a22 = G[1][1] - 2 * G[1][2] + G[2][2];
    const double b1 = G[0][0] - G[0][1], b2 = G[0][1] - G[0][2];
    const double det = a11 * a22 - a12 * a12;
    if (det > 1e-12 * a11 * a22 && a11 > 0 && a22 > 0) {
      g1 = (b1 * a22 - b2 * a12) / det;
      g2 = (a11 * b2 - a12 * b1) / det;
    } else {
      m = 1;
    }
    if (m == 2 && !(fabs(g1) < 8.0 && fabs(g2) < 8.0)) {
      g1 = g2 = 0;
      m = 1;
    }
  }
  if (m == 1) {
    const double a11 = G[0][0] - 2 * G[0][1] + G[1][1], b1 = G[0][0] - G[0][1];
    g1 = a11 > 0 ? b1 / a11 : 0.0;
    g2 = 0;
    if (!(fabs(g1) < 8.0)) g1 = 0;
  }
  coef[0] = 1.0 - g1;
  coef[1] = g1 - g2;
  coef[2] = g2;
  return (coef[1] != 0.0 || coef[2] != 0.0) ? (coef[2] != 0.0 ? 2 : 1) : 0;
}

// shifts a newest-first Gram matrix by one sweep and enters the new row
// (q_0 . q_0, q_0 . q_1, q_0 . q_2)
__device__ __forceinline__ void aa_gram_push(double (&G)[3][3], double a, double b, double c) {
  G[2][2] = G[1][1];
  G[1][2] = G[2][1] = G[0][1];
  G[1][1] = G[0][0];
  G[0][0] = a;
  G[0][1] = G[1][0] = b;
  G[0][2] = G[2][0] = c;
}

}  // namespace tbsla
