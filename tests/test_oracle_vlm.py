"""The oracle's vortex-lattice air source (restating src/VLM.cpp) against known answers: lifting-line
theory for a flat rectangular wing, mirror symmetry of the circulations, the freestream far from
the wing, the panel layout of a swept, tapered wing with a deflected flap; and the para-file
reader's VLM keys.  CPU only."""
import math

import numpy as np
import pytest

from fjsph_gb300 import _cdefs as d
from fjsph_gb300 import cases
from fjsph_gb300._lib import lib
from fjsph_gb300.settings import parse_para_text, apply_para, defaults, read_vlm


def _oracle(v_inf):
    from oracle.pyoracle import Oracle
    c = cases.droplet_3d()
    s = c.settings.copy()
    for k in range(3):
        s.v_inf[k] = v_inf[k]
    s.asource = d.VLM_INFL
    return Oracle(s, c.blocks, c.inlets)


def _wing(**kw):
    v = d.Vlm()
    lib().fjsph_vlm_defaults(v)
    for k, val in kw.items():
        setattr(v, k, val)
    return v


def test_vlm_defaults_match_reference_constructor():
    v = _wing()
    assert v.span == -1 and v.chord == -1 and v.panels_span == -1 and v.panels_chord == -1
    assert v.max_vel_fac == 2.0 and v.max_vel == 2.0 and v.taper == 0.0 and v.sweep_deg == 0.0


def test_flat_wing_lift_slope_and_symmetry():
    V, a = 50.0, math.radians(5.0)
    o = _oracle([V * math.cos(a), 0.0, V * math.sin(a)])
    v = _wing(span=10.0, chord=1.0, panels_span=20, panels_chord=6, taper=1.0)
    n = o.vlm_setup(v)
    assert n == 2 * 20 * 6
    g, abc = o.vlm_panels()
    # mirror symmetry about y = 0: strip i and strip -1-i carry the same circulations
    gs = g.reshape(40, 6)
    assert np.max(np.abs(gs - gs[::-1])) < 1e-12 * np.max(np.abs(g))
    # Kutta-Joukowski lift against Prandtl's lifting line, 2 pi a AR / (AR + 2) (elliptic loading;
    # a rectangular wing sits a few per cent below it)
    dy = abc[:, 1, 1] - abc[:, 0, 1]
    cl = 2.0 * np.sum(g * dy) / (V * 2.0 * v.span * v.chord)
    ar = 2.0 * v.span / v.chord
    cl_ll = 2.0 * math.pi * a * ar / (ar + 2.0)
    assert 0.9 * cl_ll < abs(cl) < 1.02 * cl_ll
    # freestream far upstream; faster over the suction side than under the wing
    u = o.vlm_velocity(np.array([[-1000.0, 0.0, 0.0], [0.5, 0.0, 0.3], [0.5, 0.0, -0.3]]))
    assert np.allclose(u[0], [V * math.cos(a), 0.0, V * math.sin(a)], rtol=0, atol=1e-3 * V)
    assert np.linalg.norm(u[1]) > V > np.linalg.norm(u[2])


def test_swept_tapered_flapped_layout():
    """Examples/VLM's wing: 50 x 14 panels per side, sweep 32.5 deg, taper 0.6, a 20 deg flap
    over strips 3-26 and the last 6 chordwise panels."""
    o = _oracle([89.69, 0.0, 7.8466])
    v = _wing(span=22.275, chord=8.491, panels_span=50, panels_chord=14, aoa_deg=5.0, sweep_deg=32.5, taper=0.6,
              flap_start=3, flap_width=24, flap_depth=6, flap_deg=20.0)
    n = o.vlm_setup(v)
    assert n == 2 * 50 * 14
    g, abc = o.vlm_panels()
    assert np.all(np.isfinite(g))
    A, C = abc[:, 0], abc[:, 2]
    # flat panels lie in z = 0; flap panels are deflected downwards (z < 0) behind the hinge
    flap = C[:, 2] < -1e-12
    assert flap.sum() == 2 * 24 * 6
    assert np.all(np.abs(A[~flap, 2]) == 0.0)
    # sweep: the leading edge moves aft with |y| (tan 32.5 deg)
    root, tip = np.argmin(np.abs(A[:, 1])), np.argmax(np.abs(A[:, 1]))
    assert A[tip, 0] > A[root, 0] + 0.5 * 22.275 * math.tan(math.radians(32.5))


def test_para_reader_selects_vlm_source():
    text = """SPH freestream velocity: 89.69,0,7.8466
VLM definition filename: (thisfile)
VLM wing dimensions: 22.275,8.491
VLM panel counts: 50,14
VLM sweep angle (degree): 32.5
VLM taper ratio: 0.6
VLM flap start (panels): 3
VLM flap width (panels): 24
VLM flap depth (panels): 6
VLM flap angle (degree): 20
"""
    s = defaults(3)
    extra = apply_para(s, parse_para_text(text))
    assert s.asource == d.VLM_INFL and extra["vlm_file"] == "(thisfile)"
    import tempfile, os
    with tempfile.NamedTemporaryFile("w", suffix=".para", delete=False) as f:
        f.write(text)
    try:
        v = read_vlm(f.name)
    finally:
        os.unlink(f.name)
    assert (v.span, v.chord, v.panels_span, v.panels_chord) == (22.275, 8.491, 50, 14)
    assert (v.flap_start, v.flap_width, v.flap_depth, v.flap_deg) == (3, 24, 6, 20.0)
    assert v.max_vel == 2.0 and v.max_vel_fac == 2.0
