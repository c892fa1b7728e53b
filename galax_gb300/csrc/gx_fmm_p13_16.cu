// gx_fmm_p13_16.cu -- force passes instantiated for expansion orders [13, 14, 15, 16].
#include "gx_fmm_impl.cuh"

GX_FMM_INSTANTIATE(13)
GX_FMM_INSTANTIATE(14)
GX_FMM_INSTANTIATE(15)
GX_FMM_INSTANTIATE(16)
