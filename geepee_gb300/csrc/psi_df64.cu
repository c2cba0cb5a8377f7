// df64 instantiation of the psi kernels (split from the API for parallel builds).
#include "psi_impl.cuh"

int psi_fwd_df64(const psi_impl::PsiArgs<double>& a, cudaStream_t st) { return psi_impl::launch_fwd<df64>(a, st); }
int psi_bwd_df64(const psi_impl::PsiArgs<double>& a, cudaStream_t st) { return psi_impl::launch_bwd<df64>(a, st); }
