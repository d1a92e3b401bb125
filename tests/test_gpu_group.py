"""Groups (several lattices and models swept as one CUDA graph) and the
tile-class autotuner, through the C ABI.

A group's sweep must give every handle exactly what sweeping it alone gives
(same kernels, same random streams); every tile class computes the same
arithmetic in the same order, so forcing a class or autotuning changes no
decision; and the autotuner puts the fields and random-stream positions
back, so a tuned handle continues the same Markov chain.
"""
import numpy as np
import pytest

import cases
from kapdqmc_gb300 import Initial_s
from kapdqmc_gb300.sweep import Sweeper, SweeperGroup

pytestmark = pytest.mark.gpu


def _setup(model, nchains, seed, precision="fp64"):
    sw = Sweeper(model, nchains)
    sw.set_precision(precision)
    sw.set_fields(np.stack([Initial_s(model, 60 + c) for c in range(nchains)]))
    sw.set_rng(seed)
    return sw


def _result(sw, obs):
    return sw.get_fields(), obs, [sw.green(c) for c in range(sw.nchains)]


def _same(a, b, tol=1e-12):
    (fa, oa, ga), (fb, ob, gb) = a, b
    np.testing.assert_array_equal(fa, fb)
    assert np.abs(oa - ob).max() <= tol * max(1.0, np.abs(ob).max())
    for x, y in zip(ga, gb):
        assert np.linalg.norm(x - y) <= tol * np.linalg.norm(y)


MEMBERS = [(cases.tu_square, 3, "fp64"), (cases.tv_honeycomb, 2, "fp64"),
           (cases.tuv_honeycomb, 4, "mixed"), (cases.tu_honeycomb, 2, "mixed")]


def test_group_equals_separate_sweeps():
    sweeps = 2
    alone = []
    for i, (make, n, prec) in enumerate(MEMBERS):
        with _setup(make(), n, 100 + i, prec) as sw:
            obs = sw.phy_update(sweeps, True)
            alone.append(_result(sw, obs))
    sws = [_setup(make(), n, 100 + i, prec) for i, (make, n, prec) in enumerate(MEMBERS)]
    try:
        with SweeperGroup(sws) as grp:
            obs = grp.phy_update(sweeps, True)
            # a second call replays the captured group graph
            for s in sws:
                s.set_fields(np.stack([Initial_s(s.model, 60 + c) for c in range(s.nchains)]))
            for i, s in enumerate(sws):
                s.set_rng(100 + i)
            obs2 = grp.phy_update(sweeps, True)
            for s, o, o2, ref in zip(sws, obs, obs2, alone):
                got = _result(s, o2)
                _same(got, ref)
                np.testing.assert_array_equal(o, o2)
    finally:
        for s in sws:
            s.close()


def test_group_rejects_duplicates_and_uninitialised():
    from kapdqmc_gb300._lib import KdqError
    with _setup(cases.tu_square(), 1, 1) as a:
        with pytest.raises(KdqError):
            SweeperGroup([a, a])
        with SweeperGroup([a]) as grp:
            with pytest.raises(KdqError):
                grp.sweep(1)          # kdq_init has not run
            a.init()
            grp.sweep(1)
            grp.synchronize()


@pytest.mark.parametrize("make", [cases.tv_honeycomb, cases.tu_square])
def test_every_tile_class_gives_the_same_chain(make):
    model = make()
    ref = None
    for rows in (1, 3, 6):
        with _setup(model, 2, 9) as sw:
            sw.set_tiles(rows)
            assert sw.tiles == rows
            got = _result(sw, sw.phy_update(2, True))
        if ref is None:
            ref = got
        else:
            _same(got, ref)


def test_tile_class_must_cover_the_lattice():
    from kapdqmc_gb300._lib import KdqError
    with _setup(cases.c2(), 1, 1) as sw:       # 72 sites
        with pytest.raises(KdqError):
            sw.set_tiles(1)
        sw.set_tiles(6)


def test_autotune_keeps_the_markov_chain():
    model = cases.tv_honeycomb()
    with _setup(model, 4, 21) as sw:
        ref = _result(sw, sw.phy_update(2, True))
    with _setup(model, 4, 21) as sw:
        rows, ms = sw.autotune()
        assert rows in ms and set(ms) == {1, 3, 6}
        assert ms[rows] == min(ms.values())
        got = _result(sw, sw.phy_update(2, True))
        rows2, _ = sw.autotune()              # cached for this shape
        assert rows2 == rows
    _same(got, ref)


def test_sweep_launch_shapes_give_identical_results():
    """One launch per sweep and one launch per stabilisation block run the
    same blocks in the same order per chain: fields, G and rows agree bit
    for bit."""
    model = cases.tu_honeycomb()
    fields = np.stack([Initial_s(model, 500 + c) for c in range(3)])
    out = []
    for per_sweep in (False, True):
        with Sweeper(model, 3) as sw:
            sw.set_precision("mixed")
            sw.set_sweep_launch(per_sweep)
            sw.set_fields(fields)
            sw.set_rng(9)
            obs = sw.phy_update(2, 2)
            out.append((sw.get_fields(), np.array([sw.green(c) for c in range(3)]), obs))
    np.testing.assert_array_equal(out[0][0], out[1][0])
    np.testing.assert_array_equal(out[0][1], out[1][1])
    np.testing.assert_array_equal(out[0][2], out[1][2])
