/* gpk.h - C ABI of libgpk.so, the GB300 (sm_103a) kernels behind geepee_gb300.
 *
 * Every entry point takes caller-owned DEVICE buffers (plain pointers, row-major,
 * explicit sizes), a cudaStream_t passed as void*, and returns an int status:
 *   GPK_OK (0) on success, >0 a LAPACK-style info (e.g. the failing pivot of a
 *   Cholesky), <0 an argument / support / CUDA error (see gpk_last_error()).
 * Launches are asynchronous on `stream`; nothing allocates device memory, so every
 * call can be captured in a CUDA graph.
 *
 * Precision `prec`: GPK_DF64 - buffers are float64 and the arithmetic is
 * double-float (two FP32 words, ~48-bit significand) on the FP32 pipes;
 * GPK_FP32 - buffers are float32 and the arithmetic is FP32.  Accumulated outputs
 * (sums over data points) are always float64 and are ADDED INTO (the caller zeroes
 * them first), so results of several launches can be combined.
 *
 * Hyperparameters are device pointers in the reference's log parameterisation:
 * lls2[q] = log ell_q^2 = 2*ls[q], lsf2[0] = log sf^2 = 2*sf
 * (the arguments geepee passes to compute_kernel / compute_psi_weave, e.g.
 * geepee/aep_models.py:154,194).
 */
#ifndef GPK_H
#define GPK_H

#ifdef __cplusplus
extern "C" {
#endif

#define GPK_OK 0
#define GPK_EINVAL (-1)
#define GPK_EUNSUPPORTED (-2)
#define GPK_ECUDA (-3)

#define GPK_DF64 0
#define GPK_FP32 1

/* Library version and the text of the last error on this thread. */
int gpk_version(void);
const char* gpk_last_error(void);

/* Index checks of the debug build.  A library built with -DGPK_DEBUG_BOUNDS (the build
 * script's debug_bounds option, libgpk_debug.so) checks the hot kernels' indexed accesses; an
 * index out of range sets a bit of an error word (the access then goes to element 0) and the
 * kernel completes.  Writes the OR of the words (bit 0 factor L, 1 GEMM tile staging, 2 psi
 * backward pair table / L / accumulators, 3 psi forward pair tables, 4 det backward row
 * buffer, 6 psi backward row sums) into *word and clears them; synchronous.  Returns 1 for a
 * debug build, 0 for a release build (*word = 0), <0 for a null pointer.  (No counterpart in
 * the reference; a debugging aid.) */
int gpk_debug_bounds(unsigned int* word);

/* ARD exponentiated-quadratic kernel matrix
 *   K[n,m] = sf2 * exp(-1/2 sum_d (x[n,d]-z[m,d])^2 / ell2[d])  (+ jitter if n == m)
 * x: [N,D] (row stride ldx), z: [M,D] (row stride ldz), K: [N,M] (row stride ldk).
 * Replaces geepee/kernels.py:10-22 compute_kernel(lls, lsf, x, z) (and the jittered
 * Kuu of base_models.py:454-464 when jitter > 0). */
int gpk_kern(int prec, int N, int M, int D, const void* x, int ldx, const void* z, int ldz,
             const double* lls2, const double* lsf2, double jitter, void* K, int ldk, void* stream);

/* Psi statistics of the ARD kernel under Gaussian inputs N(mu, var), fused with the
 * moment-matching contractions of one sparse-GP layer.
 *   psi1[n,m]   = sf2 prod_q sqrt(l/(l+S)) exp(-(mu-z_m)^2 / (2(l+S)))
 *   psi2[n,a,b] = sf2^2 prod_q sqrt(l/(l+2S)) exp(-(z_a-z_b)^2/(4l) - (mu-(z_a+z_b)/2)^2/(l+2S))
 * Inputs: mu, var [N,Q]; Z [M,Q]; optional A [Dout,M] and B [Dout,M,M].
 * Outputs (each optional, NULL to skip):
 *   psi1 [N,M]; psi2 [N,M,M] (full symmetric, per point); psi2_sum [M,M] += sum_n psi2
 *   (float64); m_out, v_out [N,Dout]:  m = psi1 A^T,  v = sf2 + sum_ab B[d,a,b] psi2[n,a,b] - m^2
 *   (A and B required for m_out / v_out).
 * Replaces geepee/kernels.py:181-240 compute_psi_weave and the contraction in
 * SGP_Layer._forward_prop_random_thru_cav_mm, geepee/aep_models.py:182-199
 * (base_models.py:286-307 for the posterior). */
int gpk_psi_fwd(int prec, int N, int M, int Q, int Dout, const void* mu, const void* var,
                const void* Z, const double* lls2, const double* lsf2, const void* A,
                const void* B, void* psi1, void* psi2, double* psi2_sum, void* m_out,
                void* v_out, void* stream);

/* Backward of gpk_psi_fwd's m/v outputs, recomputing psi1/psi2 (nothing N*M*M is stored).
 * Given m [N,Dout] and upstream gradients dm, dv [N,Dout]:
 *   dm_all = dm - 2 dv m;  dpsi1 = dm_all A;  dpsi2[n] = sum_d dv[n,d] B[d]
 * and returns the gradients of  sum(dpsi1*psi1) + sum(dpsi2*psi2):
 *   dsf2 [1] (w.r.t. sf^2), dl [Q] (w.r.t. ell, not ell^2), dZ [M,Q]   (+=, float64)
 *   dA [Dout,M] += sum_n dm_all[n,d] psi1[n,:];  dB [Dout,M,M] += sum_n dv[n,d] psi2[n]
 *   dmu, dvar [N,Q] (overwritten, buffer precision).
 * Replaces geepee/kernels.py:302-309 compute_psi_derivatives (psi1compDer :355-378,
 * psi2compDer :402-444) together with the dAhat/dBhat/dpsi einsums of
 * SGP_Layer.backprop_grads_lvm_mm, geepee/aep_models.py:238-245. */
int gpk_psi_bwd(int prec, int N, int M, int Q, int Dout, const void* mu, const void* var,
                const void* Z, const double* lls2, const double* lsf2, const void* A,
                const void* B, const void* m, const void* dm, const void* dv, double* dsf2,
                double* dl, double* dZ, double* dA, double* dB, void* dmu, void* dvar,
                void* stream);


/* As gpk_psi_bwd, with two generic modes used by the drop-in compute_psi_derivatives:
 *   dpsi1 != NULL : an arbitrary upstream gradient dL/dpsi1 [N,M] replaces dm_all A
 *                   (A, m, dm may then be NULL; dA is not touched);
 *   b_stride != 0 : B holds a per-point dL/dpsi2 (point n at B + n*b_stride, Dout = 1,
 *                   dv ignored, dB not touched).
 * Replaces geepee/kernels.py:302-309 for arbitrary (dL_dpsi1, dL_dpsi2). */
int gpk_psi_bwd_ex(int prec, int N, int M, int Q, int Dout, const void* mu, const void* var,
                   const void* Z, const double* lls2, const double* lsf2, const void* A,
                   const void* B, const void* m, const void* dm, const void* dv, const void* dpsi1,
                   long b_stride, double* dsf2, double* dl, double* dZ, double* dA, double* dB,
                   void* dmu, void* dvar, void* stream);

/* Deterministic-input sparse-GP layer, forward (fused):
 *   kfu = K(x, Z) [N,M];  m[n,d] = kfu_n . A_d;  Bk[n,d,b] = sum_a B[d,a,b] kfu[n,a];
 *   v[n,d] = sf2 + kfu_n . Bk[n,d]
 * x [N,D] (row stride ldx), Z [M,D], A [Dout,M], B [Dout,M,M].  kfu/Bk/m/v optional.
 * Replaces SGP_Layer._forward_prop_deterministic_thru_cav, geepee/aep_models.py:142-158
 * (and _thru_post, base_models.py:265-284). */
int gpk_det_fwd(int prec, int N, int M, int D, int Dout, const void* x, int ldx, const void* Z,
                const double* lls2, const double* lsf2, const void* A, const void* B, void* kfu,
                void* Bk, void* m_out, void* v_out, void* stream);

/* The contractions of gpk_det_fwd from given kernel values kfu [N,M] (e.g. from gpk_kern):
 *   m[n,d] = kfu_n . A_d;  Bk[n,d,b] = sum_a B[d,a,b] kfu[n,a];  v[n,d] = sf2 + kfu_n . Bk[n,d]
 * so that kfu, which needs only the inputs and the kernel hyperparameters, can be formed
 * ahead (beside the factorisations that the cavity's A and B wait for).  Needs M <= 128 and
 * Dout M^2 elements in shared memory (gpk_det_contract_supported says whether a size is
 * supported; an unsupported one returns GPK_EUNSUPPORTED).  Bk, m_out, v_out optional.
 * b_pairs != 0 (GPK_DF64 only): B holds double-float (hi, lo) float pairs, as gpk_cavity_forms
 * writes them into Bd_pair, and is read without conversion.
 * Replaces the Kfu contractions of geepee/aep_models.py:142-158 (base_models.py:265-284). */
int gpk_det_contract_supported(int prec, int M, int Dout);
int gpk_det_contract(int prec, int N, int M, int Dout, const void* kfu, const double* lsf2, const void* A,
                     const void* B, int b_pairs, void* Bk, void* m_out, void* v_out, void* stream);

/* Deterministic-input layer, backward through kfu:
 *   dkfu = dm A + 2 dv Bk   (or the given dkfu [N,M] when dkfu != NULL)
 * returns (+=, float64) dsf2 [1], dl [D] (w.r.t. ell), dZ [M,D], dA [Dout,M] += dm^T kfu,
 * and optionally dx [N,D] (overwritten).  Replaces kfucompDer / compute_kfu_derivatives,
 * geepee/kernels.py:312-313,381-399, with the dkfu einsums of aep_models.py:452-454. */
int gpk_det_bwd(int prec, int N, int M, int D, int Dout, const void* x, int ldx, const void* Z,
                const double* lls2, const double* lsf2, const void* A, const void* kfu, const void* Bk,
                const void* dm, const void* dv, const void* dkfu, double* dsf2, double* dl, double* dZ,
                double* dA, void* dx, void* stream);

/* Moment-propagation rollout through a GP layer's posterior (Q inputs -> Q outputs): T steps,
 * step t taking step t-1's output moments as its input means and variances (step 0: mu0,
 * var0 [Q]); m_out, v_out [T, Q] receive m_t = psi1 A^T and v_t = sf2 + sum_ab B psi2 - m_t^2.
 * One CTA runs the whole sequence (one launch).  The transition rollout of the GP state-space
 * model's predict_forward_mm, geepee/base_models.py:1463-1502. */
int gpk_psi_rollout(int prec, int T, int M, int Q, const void* mu0, const void* var0, const void* Z,
                    const double* lls2, const double* lsf2, const void* A, const void* B, void* m_out, void* v_out,
                    void* stream);

/* Weighted Gram reduction over rows:  C[d] += sum_n w[n,d] u_n v_n^T  (u, v [N,M], w [N,Dout],
 * C [Dout,M,M] float64).  The einsum('nd,na,nb->dab') / einsum('na,nd,nb->dab') reductions of
 * geepee/aep_models.py:464,493.  When u and v are the same buffer, C is symmetric: the tiles
 * above the diagonal are formed once and added at both positions. */
int gpk_gram(int prec, int N, int M, int Dout, const void* u, const void* v, const void* w, double* C,
             void* stream);

/* c[d] += sum_n w[n,d] u_n  (u [N,M], w [N,Dout], c [Dout,M] float64);
 * einsum('nd,nm->dm') of geepee/aep_models.py:239,463,490. */
int gpk_wsum(int prec, int N, int M, int Dout, const void* u, const void* w, double* c, void* stream);

/* Batched GEMM  C[b] = alpha op(A[b]) op(B[b]) + beta C[b]  (row-major; op = transpose when
 * transA/transB != 0; batch strides in elements, 0 broadcasts).  In the df64 precision the
 * products of the M x M AEP algebra (np.einsum chains such as 'ab,dbc,ce->dae',
 * geepee/aep_models.py:252,258, base_models.py:480-488) run on the FP32 pipes.  With k == 0,
 * C = beta C and A, B may be null. */
int gpk_gemm(int prec, int batch, int m, int n, int k, int transA, int transB, double alpha,
             const void* A, int lda, long strideA, const void* B, int ldb, long strideB, double beta,
             void* C, int ldc, long strideC, void* stream);

/* gpk_gemm with a separate addend:  C[b] = alpha op(A[b]) op(B[b]) + beta E[b]  (E may alias C;
 * strideE = 0 broadcasts one E to every batch entry).  Folds the "- Kuuinv" / "+ scale * X"
 * terms of the AEP algebra (geepee/aep_models.py:536-546) into the product's epilogue. */
int gpk_gemm_ex(int prec, int batch, int m, int n, int k, int transA, int transB, double alpha,
                const void* A, int lda, long strideA, const void* B, int ldb, long strideB, double beta,
                const void* E, int lde, long strideE, void* C, int ldc, long strideC, void* stream);

/* One product of a gpk_gemm_group: the arguments of gpk_gemm_ex, and an optional operand
 * choice made on the device: when sel != NULL and bit `selbit` of sel[b] is set, batch entry b
 * reads A2 (stride strideA2) in place of A when A2 != NULL, and B2 (stride strideB2) in place
 * of B when B2 != NULL (same shapes and leading dimensions).  E.g. the layer algebra's
 * T Suhat or Kuu^-1 Suhat, whichever the regime word of output b selects (gpk_regime).  With
 * u != NULL the epilogue also adds gamma u[b] v[b]^T (u: m elements at u + b strideU, v: n at
 * v + b strideV, storage type): the rank-one terms of the layer algebra, e.g. the
 * dAhat muhat^T beside dBhat G, without a separate linear combination. */
typedef struct {
  int batch, m, n, k, transA, transB;
  double alpha, beta;
  const void* A;
  int lda;
  long strideA;
  const void* B;
  int ldb;
  long strideB;
  const void* E;
  int lde;
  long strideE;
  void* C;
  int ldc;
  long strideC;
  const int* sel;
  int selbit;
  const void* A2;
  long strideA2;
  const void* B2;
  long strideB2;
  double gamma;
  const void* u;
  long strideU;
  const void* v;
  long strideV;
} gpk_gemm_t;
#define GPK_GEMM_GROUP 16

/* Up to GPK_GEMM_GROUP independent gpk_gemm_ex products in one launch (the products of one
 * dependency level of the AEP algebra, e.g. mu = Su theta_2 and muhat = beta Suhat theta_2 of
 * every layer).  The outputs must not overlap each other or the inputs. */
int gpk_gemm_group(int prec, int count, const gpk_gemm_t* problems, void* stream);

/* Batched SPD factorisation of A[b] (M x M, M <= 128): writes (each optional) the inverse
 * Ainv, the lower Cholesky factor L, logdet = log det A, and info[b] = 0 or the 1-based
 * pivot where A[b] stopped being positive definite (LAPACK potrf convention).
 * Replaces np.linalg.inv / slogdet on Kuu, Su^-1, Suhat^-1 (geepee/base_models.py:464,471,
 * aep_models.py:68,78,91,525). */
int gpk_chol_inv(int prec, int batch, int M, const void* A, void* Ainv, void* L, double* logdet, int* info,
                 void* stream);

/* As gpk_chol_inv for any M <= 4096: the factorisation runs in the caller's device workspace
 * `work` (batch*M*M elements of the buffer precision) instead of shared memory; required for
 * M > 128 (e.g. the M = 200 models of the serving mix). */
int gpk_chol_inv_ws(int prec, int batch, int M, const void* A, void* Ainv, void* L, double* logdet, int* info,
                    void* work, void* stream);

/* SPD inverse and log-determinant, the fast path for the AEP algebra: Ainv[b] = A[b]^-1,
 * logdet and info as in gpk_chol_inv (info is required).  For M <= 128 three launches: a
 * one-CTA register-tiled Cholesky writes L into `work`, a many-CTA column-parallel forward
 * substitution writes L^-1 after it, and the GEMM forms L^-T L^-1; for larger M the
 * factorisation runs in `work`.  `work`: 2*batch*M*M elements of the buffer precision.
 * Replaces np.linalg.inv + slogdet of Kuu, Su^-1, Suhat^-1 (geepee/base_models.py:464, 471,
 * aep_models.py:68,78,91,525). */
int gpk_spd_inv(int prec, int batch, int M, const void* A, void* Ainv, double* logdet, int* info, void* work,
                void* stream);

/* gpk_spd_inv without a workspace argument and without allocating: the workspace is a
 * file-scope device array of the library (2 MiB), so the limit is M <= 128, batch <= 65535
 * and batch*M*M <= 131072 (e.g. 8 matrices of 128 x 128); larger inputs are rejected with
 * GPK_EINVAL.  No counterpart in the reference (an interface of this library only).  The
 * array is one per device and needs no zeroing; calls that overlap on a device (other
 * streams or host threads) race on it.  The array's address is looked up on the current
 * device at every call, so `stream` must belong to the current device; the first call on a
 * device loads the library's module there and should come before any stream capture. */
int gpk_spd_inv_static(int prec, int batch, int M, const void* A, void* Ainv, double* logdet, int* info,
                       void* stream);

/* ---- fused float64 pieces of the M x M AEP algebra (no counterpart kernels in the reference:
 * each replaces a chain of numpy expressions; the arithmetic stays float64) ---- */

#define GPK_LC_TERMS 6
#define GPK_LC_RANK 3

/* out[b,i,j] = sum_t cX[t] X[t][b*sX[t] + (tX[t] ? j*cols+i : i*cols+j)]
 *            + sum_r cr[r] u[r][b*su[r] + i] v[r][b*sv[r] + j]
 * for b < batch, i < rows, j < cols (row-major).  A stride of 0 broadcasts a term over the
 * batch; tX transposes a (square) term.  With sum_batch != 0 the result is summed over b into
 * one rows x cols output (broadcast terms then enter once).  `out` may alias a term only
 * elementwise (same index, no transpose, no batch sum).  E.g. Su^-1 = Kuu^-1 + theta_1,
 * Bhat_sto = Bhat_det + Ahat Ahat^T, sum_d(...) of geepee/aep_models.py:226-304, 536-546. */
typedef struct {
  int batch, rows, cols, sum_batch;
  int nterm, nrank;
  const double* X[GPK_LC_TERMS];
  long sX[GPK_LC_TERMS];
  double cX[GPK_LC_TERMS];
  int tX[GPK_LC_TERMS];
  const double* u[GPK_LC_RANK];
  long su[GPK_LC_RANK];
  const double* v[GPK_LC_RANK];
  long sv[GPK_LC_RANK];
  double cr[GPK_LC_RANK];
  double* out;
} gpk_lincomb_t;
int gpk_lincomb(const gpk_lincomb_t* desc, void* stream);

/* The regime word of each output d of a natural-parameter layer (T = theta_1 [D,M,M],
 * K = Kuu): bit 0 set when beta max|T_d| <= max|K^-1| (the cavity is prior-dominated: its
 * moments are formed from T, as products with K^-1 would cancel), bit 1 set when
 * max|T_d| <= max|K^-1| (the same for the posterior).  flags [D] int. */
int gpk_regime(int D, int M, double beta, const double* T, const double* Kinv, int* flags, void* stream);

/* The posterior and cavity moments of a natural-parameter layer (t = theta_2 [D,M],
 * Su = (K^-1 + T)^-1, Suhat = (K^-1 + beta T)^-1) in the form its regime word selects:
 *   cavity, bit 0 set:  Bhat_det = beta^2 Qh - beta T,  Ahat = beta t - beta vh,
 *           (Qh = T Suhat T, vh = T muhat);
 *   bit 0 clear:        Bhat_det = Qh - K^-1,            Ahat = vh
 *           (Qh = K^-1 Suhat K^-1, vh = K^-1 muhat);
 *   posterior likewise with bit 1, beta = 1, Qu (T Su T or K^-1 Su K^-1), vu (T mu or K^-1 mu):
 *   B = Qu - T or Qu - K^-1,  A = t - vu or vu;
 * Bhat_sto = Bhat_det + Ahat Ahat^T, and G = K^-1 Suhat (= I - beta Ph when bit 0 is set, Ph
 * = T Suhat; = Ph = K^-1 Suhat otherwise), which the backward's algebra uses.  Bd_pair
 * (optional, D M M pairs of floats) receives Bhat_det again as double-float (hi, lo) pairs, the
 * form gpk_det_contract reads without converting.  Qh, Qu [D,M,M],
 * vh, vu [D,M] and Ph are the products of the selected form (gpk_gemm_t's sel).  Elementwise
 * float64.  The quantities of geepee/aep_models.py:536-546 and base_models.py:480-488, which
 * always take the K^-1 form. */
typedef struct {
  int D, M;
  double beta;
  const double *T, *Kinv, *t, *Qh, *Qu, *vh, *vu, *Ph;
  const int* flags;
  double *Bd, *Bp, *Bsto, *Ah, *A, *G;
  float* Bd_pair;
} gpk_forms_t;
#define GPK_FORMS_MAX 8
int gpk_cavity_forms(int n, const gpk_forms_t* items, void* stream);

/* One dependency level of the AEP algebra in one launch: up to GPK_GEMM_GROUP products (as
 * gpk_gemm_group) and up to GPK_LC_GROUP linear combinations (as gpk_lincomb), all independent
 * of each other (no output read or written by another member).  E.g. the posterior moments
 * Su + mu mu^T and Suhat + muhat muhat^T with the products K^-1 muhat and K^-1 Suhat
 * (geepee/aep_models.py:536-546).  gpk_gemm_group is this call without linear combinations. */
#define GPK_LC_GROUP 4
int gpk_level(int prec, int ngemm, const gpk_gemm_t* gemms, int nlc, const gpk_lincomb_t* lincombs, void* stream);

/* q(u) unpacking for a natural-parameter layer: R[d] = upper triangle of the packed
 * eta1_R[d] (row-major np.triu_indices order) with exp() on the diagonal, zeros below;
 * lls2 = 2 ls, lsf2 = 2 sf.  (geepee/base_models.py:630-658 update_hypers.) */
int gpk_nat_prep(int D, int M, int Q, const double* eta1, const double* ls, const double* sf, double* R,
                 double* lls2, double* lsf2, void* stream);

/* d eta1_R from dR = R (dtheta_1 + dtheta_1^T): out[d,p] (+)= dR[d,a,b] * (a == b ? R[d,a,a] : 1)
 * for the upper-triangle entry p = (a, b) (geepee/aep_models.py:274-287). */
int gpk_triu_pack(int D, int M, const double* dR, const double* R, double* out, int accumulate, void* stream);

/* Kernel hyperparameter gradients: g_ls[q] = dl[q] exp(ls[q]), g_sf = 2 exp(2 sf) (dsf2 + sum dv)
 * (geepee/aep_models.py:226-231, 445-450). */
int gpk_hyp_grads(int Q, const double* ls, const double* sf, const double* dl, const double* dsf2,
                  const double* dv, int ndv, double* g_ls, double* g_sf, void* stream);

/* *out += w * phi, the natural-parameter layer's weighted log-partition
 * phi = D/2 logdet Kuu + (N/a - 1)(-1/2 sum_d logdet Su^-1 + 1/2 mu.th2)
 *       - (N/a)(-1/2 sum_d logdet Suhat^-1 + 1/2 beta muhat.th2),  beta = (N - a)/N
 * (geepee/aep_models.py:62-114; mu.Su^-1 mu = mu.th2 since mu = Su th2). */
int gpk_aep_phi(int D, int M, double N, double alpha, const double* logdetK, const double* ldSuinv,
                const double* ldShinv, const double* mu, const double* mh, const double* th2, double w,
                double* out, void* stream);

/* Gaussian likelihood of a minibatch of n x D outputs (Gauss_Layer.compute_log_Z and
 * backprop_grads, geepee/lik_layers.py:119-181), with vt = v + exp(2 sn)/alpha, r = y - m:
 *   dm = scale r/vt,  dv = scale (-1/(2 vt) + r^2/(2 vt^2))         (written, [n, D])
 *   *energy = scale * logZ * invN,  *g_sn = scale (sum(dv)/scale * 2 sn2/alpha + n D (1-alpha)) * invN
 * (both overwritten); logZ includes the alpha-power normaliser n D (log(2 pi sn2/alpha)/2
 * - alpha log(2 pi sn2)/2).  part 0 does both; part 1 only dm, dv; part 2 only the two sums
 * (after part 1, e.g. on a second stream while the backward consumes dm, dv). */
int gpk_gauss_lik(int n, int D, const double* m, const double* v, const double* y, const double* sn, double alpha,
                  double scale, double invN, double* dm, double* dv, double* energy, double* g_sn, int part,
                  void* stream);

/* Probit likelihood of labels y in {-1, +1} (Probit_Layer.compute_log_Z,
 * geepee/lik_layers.py:303-416; the layer has no hyperparameters, so backprop_grads
 * returns nothing).  mc = 0, S = 1: the 2-D case, m, v, y [n, D].  mc = 1: the sampled
 * 3-D case, m, v [S, n, D] (S <= 16) against y [n, D], a log-mean-exp over the samples.
 * alpha == 1 is the closed form with erf; any other alpha uses T <= 16 Gauss-Hermite nodes
 * gh_x, gh_w (device float64; np.polynomial.hermite.hermgauss(T), T = 10 in the reference).
 * Writes dm, dv = scale * (dlogZ/dm, dlogZ/dv) shaped like m, work[0:n*D] (each element's
 * log-partition; caller scratch) and *out = scale * invN * logZ (overwritten).  With n = 0 only
 * out is read (it is set to 0). */
int gpk_probit_lik(int S, int n, int D, int mc, const double* m, const double* v, const double* y, double alpha,
                   int T, const double* gh_x, const double* gh_w, double scale, double invN, double* dm,
                   double* dv, double* work, double* out, void* stream);

/* Expected log-likelihood of a minibatch under q(f) = N(m, v), the data term of the
 * variational free energy, m, v, y [n, D]; with S > 1, m and v hold S samples [S, n, D] against
 * y [n, D] and every term is averaged over them (the 3-D forms of the same functions):
 *   kind 0, Gaussian (Gauss_Layer.compute_log_lik_exp, backprop_grads_log_lik_exp,
 *     geepee/lik_layers.py:183-228): *g_sn = scale * invN * sum(-1 + (y^2 - 2ym + m^2 + v)/sn2),
 *     work [2 S n D];
 *   kind 1, probit (Probit_Layer.compute_log_lik_exp, lik_layers.py:418-436) with T <= 16
 *     Gauss-Hermite nodes gh_x, gh_w (hermgauss(T)); sn and g_sn unused; work [S n D].
 * Writes dm, dv = scale * d/d(m, v) and *out = scale * invN * sum E[log p(y|f)] (overwritten). */
int gpk_lik_exp(int kind, int S, int n, int D, const double* m, const double* v, const double* y, const double* sn, int T,
                const double* gh_x, const double* gh_w, double scale, double invN, double* dm, double* dv,
                double* work, double* out, double* g_sn, void* stream);

/* Minibatch rows of two row-major float64 arrays in one launch, x[idx] and y[idx] of
 * geepee/aep_models.py:912-916 (rows = the arrays' row count): d0[i,:] = s0[idx[i],:] with c0
 * columns and d1[i,:] = s1[idx[i],:] with c1 columns (c1 = 0: none).  An index outside
 * [0, rows) gives a NaN row. */
int gpk_gather_rows(int n, long long rows, const long long* idx, int c0, const double* s0, double* d0, int c1,
                    const double* s1, double* d1, void* stream);

/* The end of an objective evaluation: g[0:span] /= divisor (grad_all[key] /= N,
 * geepee/aep_models.py:663-665, 984-986) and *worst = max(info[0:ninfo]) as a double (0, or a
 * failing Cholesky pivot of the evaluation's factorisations). */
int gpk_finish(int span, double* g, double divisor, int ninfo, const int* info, double* worst, void* stream);

/* Gradient of tr(Mm Kzz), Kzz = K(Z, Z) without jitter, w.r.t. log sf^2, log ell^2 and Z,
 * added with scales: g_sf += s_sf * d/dlog sf^2, g_ls += s_ls * d/dlog ell^2, g_z += d/dZ.
 * Replaces geepee/kernels.py:447-475 d_trace_MKzz_dhypers. */
int gpk_trace_kzz(int prec, int M, int Q, const void* Mm, const void* Z, const double* lls2,
                  const double* lsf2, double s_sf, double s_ls, double* g_sf, double* g_ls, double* g_z,
                  void* stream);

/* ---- fixed-order accumulation (bit-reproducible sums over data points) ----
 * gpk_psi_bwd_ex, gpk_det_bwd, gpk_gram and gpk_trace_kzz add per-CTA partial sums into their
 * float64 outputs with atomics, in an order that varies from run to run; the last bits of those
 * sums vary with it (and the AEP gradients propagate them through ill-conditioned M x M
 * algebra).  Each *_ws variant below takes a caller-owned float64 workspace instead: every CTA
 * writes its partial sums there, and a second launch on the same stream adds them into the
 * outputs in a fixed order (float64 additions), one writer per output element, so
 * repeated calls on the same inputs give bit-identical outputs.  work = NULL gives the atomic
 * form.  gpk_work_elems gives the workspace size in float64 elements for operation `op` at the
 * given sizes on the current device (N rows; D = Q input dimensions; Dout outputs); it may
 * exceed what one call uses.  No counterpart in the reference (numpy's sums are sequential). */
#define GPK_OP_PSI_BWD 1
#define GPK_OP_DET_BWD 2
#define GPK_OP_GRAM 3
#define GPK_OP_TRACE_KZZ 4
int gpk_work_elems(int op, int N, int M, int D, int Dout, long* elems);
int gpk_psi_bwd_ws(int prec, int N, int M, int Q, int Dout, const void* mu, const void* var,
                   const void* Z, const double* lls2, const double* lsf2, const void* A,
                   const void* B, const void* m, const void* dm, const void* dv, const void* dpsi1,
                   long b_stride, double* dsf2, double* dl, double* dZ, double* dA, double* dB,
                   void* dmu, void* dvar, double* work, long work_elems, void* stream);
int gpk_det_bwd_ws(int prec, int N, int M, int D, int Dout, const void* x, int ldx, const void* Z,
                   const double* lls2, const double* lsf2, const void* A, const void* kfu, const void* Bk,
                   const void* dm, const void* dv, const void* dkfu, double* dsf2, double* dl, double* dZ,
                   double* dA, void* dx, double* work, long work_elems, void* stream);
int gpk_gram_ws(int prec, int N, int M, int Dout, const void* u, const void* v, const void* w, double* C,
                double* work, long work_elems, void* stream);
int gpk_trace_kzz_ws(int prec, int M, int Q, const void* Mm, const void* Z, const double* lls2,
                     const double* lsf2, double s_sf, double s_ls, double* g_sf, double* g_ls, double* g_z,
                     double* work, long work_elems, void* stream);

/* Batched inverse and log-determinant of many tiny SPD matrices A[b] (n x n, n <= 8), one
 * thread per matrix; info[b] as in gpk_chol_inv.  Replaces the per-time-step
 * np.linalg.solve / inv / slogdet of Gauss_Emis.compute_emission_tilted,
 * geepee/lik_layers.py:596-610. */
int gpk_small_spd(int prec, int batch, int n, const void* A, void* Ainv, double* logdet, int* info,
                  void* stream);

#ifdef __cplusplus
}
#endif
#endif /* GPK_H */
