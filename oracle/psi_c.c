/* Plain C restatement of the reference's psi-statistics loop (geepee/kernels.py:201-234)
 * fused with the moment-matching contraction of aep_models.py:193-198.
 * TEST INFRASTRUCTURE ONLY: the scalar CPU baseline and a checker; never linked into
 * the product.  Single-threaded, float64.
 *
 *   psi1[n,m]   = sf2 exp(sum_q -(mu-z_m)^2/(2(l+S)) + 1/2 log(l/(l+S)))
 *   psi2[n,a,b] = sf2^2 exp(sum_q -(z_a-z_b)^2/(4l) - (mu-(z_a+z_b)/2)^2/(l+2S) + 1/2 log(l/(l+2S)))
 *   m[n,d] = sum_a psi1 A[d,a];  v[n,d] = sf2 + sum_ab B[d,a,b] psi2[n,a,b] - m^2
 *   psi2_sum[a,b] += sum_n psi2[n,a,b]  (if non-NULL)
 */
#include <math.h>
#include <stddef.h>

void oracle_psi_fwd(int N, int M, int Q, int Dout, const double* mu, const double* S, const double* Z,
                    const double* ell2, double sf2, const double* A, const double* B, double* m_out,
                    double* v_out, double* psi2_sum) {
  double ld1[64], ld2[64];
  double psi1[1024];
  for (int n = 0; n < N; ++n) {
    const double* mun = mu + (size_t)n * Q;
    const double* Sn = S + (size_t)n * Q;
    for (int q = 0; q < Q; ++q) {
      ld1[q] = 0.5 * log(ell2[q] / (ell2[q] + Sn[q]));
      ld2[q] = 0.5 * log(ell2[q] / (ell2[q] + 2.0 * Sn[q]));
    }
    for (int a = 0; a < M; ++a) {
      double e = 0.0;
      for (int q = 0; q < Q; ++q) {
        double d = mun[q] - Z[a * Q + q];
        e += -d * d / 2.0 / (Sn[q] + ell2[q]) + ld1[q];
      }
      psi1[a] = sf2 * exp(e);
    }
    double vacc[16] = {0};
    for (int a = 0; a < M; ++a) {
      for (int b = 0; b <= a; ++b) {
        double e = 0.0;
        for (int q = 0; q < Q; ++q) {
          double za = Z[a * Q + q], zb = Z[b * Q + q];
          double mh = mun[q] - (za + zb) / 2.0;
          double dz = za - zb;
          e += -dz * dz / (4.0 * ell2[q]) - mh * mh / (2.0 * Sn[q] + ell2[q]) + ld2[q];
        }
        double p = sf2 * sf2 * exp(e);
        if (psi2_sum) {
          psi2_sum[a * M + b] += p;
          if (a != b) psi2_sum[b * M + a] += p;
        }
        for (int d = 0; d < Dout; ++d) {
          const double* Bd = B + (size_t)d * M * M;
          vacc[d] += (a == b ? Bd[a * M + a] : Bd[a * M + b] + Bd[b * M + a]) * p;
        }
      }
    }
    for (int d = 0; d < Dout; ++d) {
      double mm = 0.0;
      for (int a = 0; a < M; ++a) mm += psi1[a] * A[d * M + a];
      if (m_out) m_out[(size_t)n * Dout + d] = mm;
      if (v_out) v_out[(size_t)n * Dout + d] = sf2 + vacc[d] - mm * mm;
    }
  }
}
