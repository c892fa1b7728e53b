// gx_fmm_p5_6.cu -- force passes instantiated for expansion orders [5, 6].
#include "gx_fmm_impl.cuh"

GX_FMM_INSTANTIATE(5)
GX_FMM_INSTANTIATE(6)
