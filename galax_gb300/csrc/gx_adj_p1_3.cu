// gx_adj_p1_3.cu -- force VJP instantiated for expansion orders 1 2 3.
#include "gx_adjoint_impl.cuh"

GX_ADJ_INSTANTIATE(0)
GX_ADJ_INSTANTIATE(1)
GX_ADJ_INSTANTIATE(2)
GX_ADJ_INSTANTIATE(3)
