// gx_adj_p4.cu -- force VJP instantiated for expansion orders 4.
#include "gx_adjoint_impl.cuh"

GX_ADJ_INSTANTIATE(4)
