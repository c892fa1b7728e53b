// gx_adj_p5_8.cu -- force VJP instantiated for expansion orders 5 6 8.
#include "gx_adjoint_impl.cuh"

GX_ADJ_INSTANTIATE(5)
GX_ADJ_INSTANTIATE(6)
GX_ADJ_INSTANTIATE(7)
GX_ADJ_INSTANTIATE(8)
