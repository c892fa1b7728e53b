// gx_fmm_p9_12.cu -- force passes instantiated for expansion orders [9, 10, 11, 12].
#include "gx_fmm_impl.cuh"

GX_FMM_INSTANTIATE(9)
GX_FMM_INSTANTIATE(10)
GX_FMM_INSTANTIATE(11)
GX_FMM_INSTANTIATE(12)
