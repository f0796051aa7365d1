"""The oracle's restatement of update_data (src/Integration.cpp:109-226, src/shapes/inlet.cpp:578-640)
on the live-inlet jet: one step inserts one BUFFER particle per column, turns every BACK particle
into PIPE and the first BUFFER particle of every column into BACK, and deletes the top layer."""
import numpy as np
import pytest

from fjsph_gb300 import _cdefs as d
from fjsph_gb300 import cases


@pytest.fixture(scope="module", autouse=True)
def _libs(oracle_lib):
    return oracle_lib


def _one_step(max_points=None):
    from oracle.pyoracle import Oracle
    c = cases.jet_inlet(pipe_layers=6, column_layers=6, max_points=max_points)
    o = Oracle(c.settings, c.blocks, c.inlets)
    o.set_states(c.state, c.state)
    o.integrate()
    return c, o


def test_insertion_and_deletion_bookkeeping():
    c, o = _one_step()
    inl = c.inlets[0]
    nd = len(inl.back)
    depth = inl.buffer.shape[1]
    st0 = c.state
    st = o.download()
    top = st0.xi[:, 2] > c.blocks[-1].delconst
    n_del = int(np.count_nonzero(top))
    assert n_del == nd                       # the top layer
    assert o.deleted() == n_del
    assert st.n == st0.n + nd - n_del
    nb = c.blocks[0].second
    assert o.limits() == [(0, nb), (nb, st.n)]
    # deleted particles (highest z, lowest indices of the top layer) are gone; ids continue
    kept_ids = np.setdiff1d(st0.part_id, st0.part_id[top])
    new_ids = np.arange(st0.n, st0.n + nd)
    np.testing.assert_array_equal(np.sort(st.part_id), np.sort(np.concatenate([kept_ids, new_ids])))
    by_id = {pid: i for i, pid in enumerate(st.part_id)}
    # old BACK -> PIPE, first buffer -> BACK, new particles BUFFER one dx below the old last
    for ii in range(nd):
        assert st.b[by_id[st0.part_id[inl.back[ii]]]] == d.PIPE
        assert st.b[by_id[st0.part_id[inl.buffer[ii, 0]]]] == d.BACK
        new = by_id[st0.n + ii]
        last = by_id[st0.part_id[inl.buffer[ii, depth - 1]]]
        assert st.b[new] == d.BUFFER
        np.testing.assert_allclose(st.xi[new], st.xi[last] - np.array([0.0, 0.0, c.settings.dx]), atol=1e-15)
    back, buf = o.get_inlet(inl.block, nd, depth)
    np.testing.assert_array_equal(st.part_id[back], st0.part_id[inl.buffer[:, 0]])
    np.testing.assert_array_equal(st.part_id[buf[:, -1]], new_ids)
    np.testing.assert_array_equal(st.part_id[buf[:, :-1]], st0.part_id[inl.buffer[:, 1:]])


def test_max_points_caps_insertion():
    c0 = cases.jet_inlet(pipe_layers=6, column_layers=6)
    c, o = _one_step(max_points=c0.state.n + 10)
    st = o.download()
    nd = len(c.inlets[0].back)
    assert st.n == c.state.n + 10 - nd      # 10 inserted, the top layer deleted
    # every column still advanced
    by_id = {pid: i for i, pid in enumerate(st.part_id)}
    assert all(st.b[by_id[c.state.part_id[i]]] == d.PIPE for i in c.inlets[0].back)
