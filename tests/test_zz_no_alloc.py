"""The allocation-free PoissonRHS entry point (cvb_poisson_rhs_noalloc).

It exists for callers that cannot call cudaMalloc -- code inside a CUDA graph
capture, hosts whose device memory comes from their own pool, time loops that
forbid allocation after start-up -- and keeps its only scratch in a fixed
file-scope device array.  Checked here through the C ABI against the regular
entry point, on two calls in a row (the second sees the scratch the first left).
This file is collected last so a failure here comes after every other test.
"""
import ctypes

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def test_noalloc_rhs_matches_regular_entry_point():
    import torch

    from cases import build
    from curvib_old_gb300 import _lib
    from curvib_old_gb300.solver import PoissonContext
    import types

    c = build("box_sphere")
    P = types.SimpleNamespace(metrics=c["metrics"], nvert=c["nvert"], bctype=c["bctype"], semi=c["semi"])
    ctx = PoissonContext().setup(P)
    mz, my, mx = c["nvert"].shape
    dev = torch.device("cuda", 0)
    d_aj = torch.tensor(c["metrics"][-1]["Aj"], dtype=torch.float64, device=dev).contiguous()
    d_nv = torch.tensor(c["nvert"], dtype=torch.float64, device=dev).contiguous()
    L = _lib.lib()
    for call, (dt, st, scale) in enumerate(((1e-3, 1.0, 1.0), (2e-3, 0.5, -3.0))):
        uc = np.ascontiguousarray(c["ucont"] * scale)
        b_ref, s_ref = ctx.poisson_rhs(uc, dt, st)
        d_uc = torch.tensor(uc, dtype=torch.float64, device=dev).contiguous()
        d_b = torch.full((mz, my, mx), float("nan"), dtype=torch.float64, device=dev)
        d_s = torch.full((1,), float("nan"), dtype=torch.float64, device=dev)
        stream = torch.cuda.current_stream(dev).cuda_stream
        rc = L.cvb_poisson_rhs_noalloc(d_uc.data_ptr(), d_aj.data_ptr(), d_nv.data_ptr(), mx, my, mz, dt, st,
                                       d_b.data_ptr(), d_s.data_ptr(), ctypes.c_void_p(stream))
        assert rc == 0, rc
        torch.cuda.synchronize()
        b = d_b.cpu().numpy()
        s = float(d_s.cpu()[0])
        assert np.array_equal(b, b_ref), f"call {call}: b differs"
        assert abs(s - s_ref) <= 1e-12 * max(1.0, np.abs(b_ref / c["metrics"][-1]["Aj"]).sum() * dt), \
            f"call {call}: compatibility sum {s} vs {s_ref}"
    # a box beyond the stated maximum is refused without touching the outputs
    big = int(_lib.lib().cvb_poisson_rhs_noalloc(d_uc.data_ptr(), d_aj.data_ptr(), d_nv.data_ptr(), 1024, 1024, 128,
                                                 1e-3, 1.0, d_b.data_ptr(), d_s.data_ptr(), None))
    assert big == _lib.CVB_BAD_INPUT
    ctx.close()
