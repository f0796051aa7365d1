"""The allocation-free time-step bound (fjsph_find_timestep_noalloc) against fjsph_find_timestep.

The no-allocation entry point exists for callers whose device memory belongs to someone else's
allocator (or who may not allocate on their time-step path): they hand in device arrays they
already own and get the time step back without the library calling cudaMalloc.  This test owns
its device arrays through torch, as such a caller would, and checks two calls in a row against
the context entry point on the same particle state.  The file is named to be collected last.
"""
import ctypes as C

import numpy as np
import pytest

from fjsph_gb300 import _cdefs as d
from fjsph_gb300 import cases

pytestmark = pytest.mark.gpu


def _dev(torch, a):
    return torch.from_numpy(np.ascontiguousarray(a, dtype=np.float64)).cuda()


@pytest.mark.parametrize("ale", [False, True])
def test_noalloc_timestep_matches_context(built_lib, ale):
    torch = pytest.importorskip("torch")
    from fjsph_gb300 import _lib
    from fjsph_gb300.api import Context

    c = cases.dam_break_3d(dx=0.03, column=(0.3, 0.3, 0.6), tank=(0.8, 0.3, 0.6), ale=ale)
    ctx = Context(c.settings, c.state.n, c.blocks)
    ctx.set_states(c.state, c.state)
    for _ in range(2):
        ctx.integrate()
    st = ctx.download()
    s = ctx.settings
    dt_ref = ctx.find_timestep()
    rep = ctx.step_report()
    nb = c.state.n - c.n_fluid
    nf = c.n_fluid

    keep = []  # device arrays stay alive while their pointers are in use

    def vec(name):
        arr = (C.POINTER(C.c_double) * 3)()
        for k in range(3):
            if k < st.dim:
                t = _dev(torch, getattr(st, name)[nb:, k])
                keep.append(t)
                arr[k] = C.cast(C.c_void_p(t.data_ptr()), C.POINTER(C.c_double))
        return arr

    def scal(name):
        t = _dev(torch, getattr(st, name)[nb:])
        keep.append(t)
        return C.cast(C.c_void_p(t.data_ptr()), C.POINTER(C.c_double))

    acc, Af, v, vPert = vec("acc"), vec("Af"), vec("v"), vec("vPert")
    Rrho, rho, curve = scal("Rrho"), scal("rho"), scal("curve")
    torch.cuda.synchronize()
    lib = _lib.lib()
    for call in range(2):
        dt = C.c_double()
        red = (C.c_double * 7)()
        rc = lib.fjsph_find_timestep_noalloc(C.byref(s), nf, acc, Af, Rrho, rho, curve, v, vPert, None,
                                             C.byref(dt), red)
        assert rc == d.OK, f"call {call}: {lib.fjsph_status_string(rc)}"
        assert dt.value == pytest.approx(dt_ref, rel=1e-12), f"call {call}"
        assert red[0] == pytest.approx(rep["maxf"], rel=1e-12)
        assert red[1] == pytest.approx(rep["maxAf"], rel=1e-12)
        assert 100.0 * red[3] / s.rho_rest == pytest.approx(rep["maxRho_pc"], rel=1e-12)
    # the stated maximum size is enforced
    dt = C.c_double()
    red = (C.c_double * 7)()
    rc = lib.fjsph_find_timestep_noalloc(C.byref(s), (1 << 24) + 1, acc, Af, Rrho, rho, curve, v, vPert, None,
                                         C.byref(dt), red)
    assert rc == d.E_CAPACITY
