// f32 instantiation of the psi forward kernels (one translation unit per kernel family
// and precision, so the build compiles them in parallel).
#include "psi_impl.cuh"

int psi_fwd_f32(const psi_impl::PsiArgs<float>& a, cudaStream_t st) { return psi_impl::launch_fwd<float>(a, st); }

// the translation unit's bounds word (debug build; 0 otherwise)
GPK_BOUNDS_READER(psi_fwd_f32)
