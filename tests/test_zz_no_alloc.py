"""The allocation-free time-step bound (fjsph_find_timestep_noalloc) against fjsph_find_timestep.

The no-allocation entry point exists for callers whose device memory belongs to someone else's
allocator (or who may not allocate on their time-step path): they hand in device arrays they
already own and get the time step back without the library calling cudaMalloc.  This test owns
its device arrays through torch, as such a caller would, and checks two calls in a row against
the context entry point on the same particle state: the time step and all seven maxima must be
bit-identical.  The file is named to be collected last.
"""
import ctypes as C
import math

import numpy as np
import pytest

from fjsph_gb300 import _cdefs as d
from fjsph_gb300 import cases

pytestmark = pytest.mark.gpu

EPS = 2.220446049250313e-16


def _dev(torch, a):
    return torch.from_numpy(np.ascontiguousarray(a, dtype=np.float64)).cuda()


def _status(lib, rc):
    return lib.fjsph_status_string(rc).decode()


def _call(lib, s, nf, ptrs):
    dt = C.c_double()
    red = (C.c_double * 7)()
    rc = lib.fjsph_find_timestep_noalloc(C.byref(s), nf, *ptrs, None, C.byref(dt), red)
    return rc, dt.value, list(red)


def _device_fields(torch, st, nb, keep):
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
    return [acc, Af, scal("Rrho"), scal("rho"), scal("curve"), v, vPert]


def _case(dim, ale):
    if dim == 2:
        return cases.dam_break_2d(dx=0.04, column=(0.4, 0.8), tank=(1.2, 1.0))
    return cases.dam_break_3d(dx=0.03, column=(0.3, 0.3, 0.6), tank=(0.8, 0.3, 0.6), ale=ale)


@pytest.mark.parametrize("dim,ale", [(2, False), (3, False), (3, True)])
def test_noalloc_timestep_matches_context(built_lib, dim, ale):
    torch = pytest.importorskip("torch")
    from fjsph_gb300 import _lib
    from fjsph_gb300.api import Context

    c = _case(dim, ale)
    ctx = Context(c.settings, c.state.n, c.blocks)
    ctx.set_states(c.state, c.state)
    for _ in range(2):
        ctx.integrate()
    st = ctx.download()
    s = ctx.settings
    # a fresh context on the same state: its maxShift is this state's alone, as the entry
    # point's is (the integrating context keeps a running maximum over its calls)
    ref = Context(s, st.n, c.blocks)
    ref.set_states(st, st)
    dt_ref = ref.find_timestep()
    max_ref = ref.timestep_maxima()
    nb = st.n - c.n_fluid
    keep = []  # device arrays stay alive while their pointers are in use
    ptrs = _device_fields(torch, st, nb, keep)
    torch.cuda.synchronize()
    lib = _lib.lib()
    for call in range(2):
        rc, dt, red = _call(lib, s, c.n_fluid, ptrs)
        assert rc == d.OK, f"call {call}: {_status(lib, rc)}"
        assert dt == dt_ref, f"call {call}: dt {dt!r} != {dt_ref!r}"
        for k in range(6):
            assert red[k] == max_ref[k], f"call {call}: maximum {k}: {red[k]!r} != {max_ref[k]!r}"
        if ale:
            assert red[6] > EPS and red[6] == max_ref[6], f"call {call}: maxShift"
        else:
            assert red[6] == 0.0
    # the stated maximum size is enforced
    rc, _, _ = _call(lib, s, (1 << 24) + 1, ptrs)
    assert rc == d.E_CAPACITY, _status(lib, rc)


def test_noalloc_timestep_without_fluid(built_lib):
    """No fluid particles: the reference's initial maxima (epsilon, 9999999) and their time step."""
    from fjsph_gb300 import _lib

    c = _case(3, False)
    s = c.settings
    lib = _lib.lib()
    null3 = (C.POINTER(C.c_double) * 3)()
    ptrs = [null3, null3, None, None, None, null3, null3]
    for call in range(2):
        rc, dt, red = _call(lib, s, 0, ptrs)
        assert rc == d.OK, f"call {call}: {_status(lib, rc)}"
        assert red == [EPS, EPS, EPS, EPS, 9999999.0, EPS, 0.0]
        H = s.H
        fac = [0.25 * math.sqrt(H / EPS), 2 * H / EPS, 0.125 * s.H_sq * s.rho_rest / s.mu, 0.067 * 9999999.0,
               0.5 * math.sqrt(H / EPS), 1.5 * H / s.speed_sound]
        safe_dt = 0.75 * min(fac)
        want = s.cfl * safe_dt
        want = min(max(want, s.delta_t_min), s.delta_t_max)
        if want > s.last_frame_time + s.frame_time_interval - s.current_time:
            want = s.last_frame_time + s.frame_time_interval - s.current_time + s.delta_t_min
        assert dt == want
