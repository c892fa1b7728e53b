// gx_fmm_p0_3.cu -- force passes instantiated for expansion orders [0, 1, 2, 3].
#include "gx_fmm_impl.cuh"

GX_FMM_INSTANTIATE(0)
GX_FMM_INSTANTIATE(1)
GX_FMM_INSTANTIATE(2)
GX_FMM_INSTANTIATE(3)
