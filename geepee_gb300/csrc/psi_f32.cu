// f32 instantiation of the psi kernels (split from the API for parallel builds).
#include "psi_impl.cuh"

int psi_fwd_f32(const psi_impl::PsiArgs<float>& a, cudaStream_t st) { return psi_impl::launch_fwd<float>(a, st); }
int psi_bwd_f32(const psi_impl::PsiArgs<float>& a, cudaStream_t st) { return psi_impl::launch_bwd<float>(a, st); }
