"""The C-ABI library loads, exports every symbol include/fjsph_gb300.h declares, and its host-only
entry points (settings defaults and Set_Values derivations) work without a GPU."""
import ctypes as C
import math
import re
from pathlib import Path

import pytest

from fjsph_gb300 import _cdefs as d

ROOT = Path(__file__).resolve().parent.parent


def test_exports_every_declared_symbol(built_lib):
    header = (ROOT / "include" / "fjsph_gb300.h").read_text()
    names = sorted(set(re.findall(r"^(?:int|const char \*)\s*(fjsph_[a-z0-9_]+)\s*\(", header, re.M)))
    assert len(names) > 30
    h = C.CDLL(str(built_lib))
    missing = [n for n in names if not hasattr(h, n)]
    assert not missing, missing


def test_abi_sizes(built_lib):
    from fjsph_gb300 import _lib
    _lib.lib()  # raises on mismatch


@pytest.mark.parametrize("dim", [2, 3])
def test_set_values(built_lib, dim):
    from fjsph_gb300 import settings as S
    s = S.defaults(dim)
    assert s.solver_type == d.NEWMARK_BETA and s.st_model == d.ST_PAIRWISE
    s.particle_step = 0.01
    s.H_fac = 1.3
    s.speed_sound = 62.64
    S.derive(s)
    H = 1.3 * 0.01
    assert s.H == pytest.approx(H)
    assert s.sr == pytest.approx(4 * H * H)
    assert s.B == pytest.approx(1000.0 * 62.64 ** 2 / 7.0)
    wc = 7 / (4 * math.pi * H * H) if dim == 2 else 21 / (16 * math.pi * H ** 3)
    assert s.W_correc == pytest.approx(wc)
    assert s.dsph_cont == pytest.approx(2 * 0.1 * H * 62.64)
    assert s.sim_mass == pytest.approx(1000.0 * 0.01 ** dim)
    assert s.rho_max == pytest.approx(1500.0) and s.rho_min == pytest.approx(500.0)
    assert s.A_plate == pytest.approx(0.01 ** (dim - 1))
    # get_n_full (src/Geometry.cpp:282-308): lattice walked from -2(H+dx) by accumulated steps
    lim = 2 * (H + 0.01)
    pts = []
    x = -lim
    while x <= lim:
        pts.append(x)
        x += 0.01
    cnt = 0
    for a in pts:
        for b in pts:
            if dim == 2:
                cnt += (a * a + b * b) < 4 * H * H
            else:
                cnt += sum((a * a + b * b + c * c) < 4 * H * H for c in pts)
    assert s.n_full == cnt


def test_rejects_variants_the_reference_cannot_build(built_lib):
    from fjsph_gb300 import _lib, settings as S
    s = S.defaults(3)
    s.particle_step = 0.01
    S.derive(s)
    s.variant = d.VAR_NOFROZEN | d.VAR_LINEAR
    h = C.c_void_p()
    assert _lib.lib().fjsph_ctx_create(C.byref(s), 100, C.byref(h)) == d.E_UNSUPPORTED
    s.variant = 0
    s.dim = 4
    assert _lib.lib().fjsph_ctx_create(C.byref(s), 100, C.byref(h)) == d.E_ARG


def test_status_strings(built_lib):
    from fjsph_gb300 import _lib
    assert _lib.lib().fjsph_status_string(d.E_CAPACITY) == b"particle count above context capacity"
