"""The allocation-free PoissonRHS entry point (cvb_poisson_rhs_noalloc).

Some callers cannot call cudaMalloc: a host whose device memory is handed out by
its own allocator or pool (PETSc's, or a framework's) that must not be bypassed,
and a time-stepping loop that forbids allocation after start-up so that a long
run cannot fail half-way on memory.  The entry point takes the caller's device
arrays and keeps its only scratch in a fixed file-scope device array.

Checked here through the C ABI on two calls in a row (the second sees the
scratch the first left): the right-hand side bit for bit and the compatibility
sum exactly against the regular entry point (same kernels, same reduction
tree), and both against the CPU oracle (b bit for bit; the sum, which the
oracle adds in another order, within 1e-12 of its scale).  This file is
collected last so a failure here comes after every other test.
"""
import ctypes
import types

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("name", ["box_sphere", "channel_periodic"])
def test_noalloc_rhs_matches_regular_entry_point_and_oracle(name):
    import torch

    from cases import build
    from curvib_old_gb300 import _lib
    from curvib_old_gb300.solver import PoissonContext
    from oracle import oracle as O

    c = build(name)
    P = types.SimpleNamespace(metrics=c["metrics"], nvert=c["nvert"], bctype=c["bctype"], semi=c["semi"])
    ctx = PoissonContext().setup(P)
    L = O.OLevel(c["metrics"][-1], c["nvert"], c["bctype"], c["semi"])
    aj = c["metrics"][-1]["Aj"]
    mz, my, mx = c["nvert"].shape
    dev = torch.device("cuda", 0)
    d_aj = torch.tensor(aj, dtype=torch.float64, device=dev).contiguous()
    d_nv = torch.tensor(c["nvert"], dtype=torch.float64, device=dev).contiguous()
    lib = _lib.lib()
    for call, (dt, st, scale) in enumerate(((1e-3, 1.0, 1.0), (2e-3, 0.5, -3.0))):
        uc = np.ascontiguousarray(c["ucont"] * scale)
        b_ref, s_ref = ctx.poisson_rhs(uc, dt, st)
        b_o, s_o = O.poisson_rhs(L, uc, dt, st)
        d_uc = torch.tensor(uc, dtype=torch.float64, device=dev).contiguous()
        d_b = torch.full((mz, my, mx), float("nan"), dtype=torch.float64, device=dev)
        d_s = torch.full((1,), float("nan"), dtype=torch.float64, device=dev)
        stream = torch.cuda.current_stream(dev).cuda_stream
        rc = lib.cvb_poisson_rhs_noalloc(d_uc.data_ptr(), d_aj.data_ptr(), d_nv.data_ptr(), mx, my, mz, dt, st,
                                         d_b.data_ptr(), d_s.data_ptr(), ctypes.c_void_p(stream))
        assert rc == 0, rc
        torch.cuda.synchronize()
        b = d_b.cpu().numpy()
        s = float(d_s.cpu()[0])
        assert np.array_equal(b, b_ref), f"call {call}: b differs from cvb_poisson_rhs"
        assert s == s_ref, f"call {call}: compatibility sum {s!r} vs {s_ref!r}"
        assert np.array_equal(b, b_o), f"call {call}: b differs from the oracle"
        assert abs(s - s_o) <= 1e-12 * max(1.0, np.abs(b_o / aj).sum() * dt), \
            f"call {call}: compatibility sum {s} vs oracle {s_o}"
    # a box beyond the stated maximum is refused without touching the outputs
    before = d_b.cpu().numpy()
    big = int(lib.cvb_poisson_rhs_noalloc(d_uc.data_ptr(), d_aj.data_ptr(), d_nv.data_ptr(), 1024, 1024, 128,
                                          1e-3, 1.0, d_b.data_ptr(), d_s.data_ptr(), None))
    assert big == _lib.CVB_BAD_INPUT
    torch.cuda.synchronize()
    assert np.array_equal(d_b.cpu().numpy(), before)
    ctx.close()
