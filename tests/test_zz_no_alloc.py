"""The allocation-free entry point gx_n2_sampled_static, called through the C ABI,
against the context entry point gx_n2_sampled and against the CPU oracle's exact
sampled sum on the same bodies.

gx_n2_sampled_static exists for callers that cannot allocate device memory when
they want a force check -- their device memory belongs to another runtime's
caching allocator, which may hold nearly all of HBM -- so it takes the caller's
device arrays and stages its indices and results through a file-scope device
array instead of allocating.  This file is collected last, and the test passes
both alone in a fresh process and after the other tests.
"""
import numpy as np
import pytest

from helpers import rel_vec_err

pytestmark = pytest.mark.gpu


def test_static_entry_point_matches_context_entry_point_and_oracle(G, oracle):
    torch = pytest.importorskip("torch")
    from galax_gb300 import presets
    O = oracle
    n = 20_000
    b = presets.plummer(n, seed=41)
    eps = 0.02
    ctx = G.GpuContext(G.GpuConfig(max_n=n, max_nodes=1 << 20, p=4, eps64=eps))
    ctx.upload_bodies(b)
    dev = [torch.from_numpy(a.copy()).to("cuda") for a in (b.x, b.y, b.mass)]
    torch.cuda.synchronize()
    stream = torch.cuda.current_stream().cuda_stream
    rng = np.random.default_rng(5)
    for call in range(2):  # two calls in a row: the shared staging array is reused
        idx = rng.choice(n, 1000 + 500 * call, replace=False)
        ax, ay = G.n2_sampled_static(dev[0].data_ptr(), dev[1].data_ptr(), dev[2].data_ptr(), n, eps, idx, stream)
        # the exact sum of the CPU oracle (an independent implementation) ...
        ox, oy = O.n2_sampled(b.x, b.y, b.mass, eps, idx)
        err_o = rel_vec_err(ax, ay, ox, oy)
        assert err_o.max() < 1e-10, (call, err_o.max())
        # ... and the context entry point on the library's own copy of the bodies
        rx, ry = ctx.n2_sampled(idx)
        err = rel_vec_err(ax, ay, rx, ry)
        assert err.max() < 1e-10, (call, err.max())
    with pytest.raises(G.GpuError) as e:
        G.n2_sampled_static(dev[0].data_ptr(), dev[1].data_ptr(), dev[2].data_ptr(), n, eps,
                            np.arange(G.N2_STATIC_MAX_SAMPLES + 1) % n, stream)
    assert e.value.code == 6
    ctx.close()
