// gx_fmm_p4.cu -- force passes instantiated for expansion orders [4].
#include "gx_fmm_impl.cuh"

GX_FMM_INSTANTIATE(4)
