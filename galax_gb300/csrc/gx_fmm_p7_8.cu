// gx_fmm_p7_8.cu -- force passes instantiated for expansion orders [7, 8].
#include "gx_fmm_impl.cuh"

GX_FMM_INSTANTIATE(7)
GX_FMM_INSTANTIATE(8)
