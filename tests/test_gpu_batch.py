"""Batched ensemble: one persistent launch per kernel position over many
uneven grids must give the per-grid results (same kernel bodies; the compiler
may contract multiply-adds differently in the batched kernels, so agreement is
to rounding, checked at 1e-13), and each grid must match the CPU oracle."""
import numpy as np
import pytest

from emix_gb300 import fields as F
from helpers import assert_close

pytestmark = pytest.mark.gpu


def _grids(sgs=1):
    ws = F.ensemble(ngrids=5, seed=11, sizes=(16, 24, 32))
    for w in ws:
        w.sgs_model = sgs
    return ws


@pytest.mark.parametrize("sgs", [1, 2])
def test_batched_equals_per_grid(emix, sgs):
    ws = _grids(sgs)
    b = emix.Batch(ws)
    b.step_per_grid(2)
    ref = [b.download(g) for g in range(len(ws))]
    for tuning in [(1, 32, 2), (4, 64, 4), (4, 128, 8), (2, 32, 0)]:
        b.upload()
        b.set_tuning(*tuning)
        b.step(2, use_graph=(tuning[0] == 4))
        for g in range(len(ws)):
            um, phi = b.download(g)
            assert_close(um, ref[g][0], tol=1e-13, what=f"grid {g} um, tuning {tuning}")
            assert_close(phi, ref[g][1], tol=1e-13, what=f"grid {g} phi, tuning {tuning}")
    b.close()


@pytest.mark.parametrize("use_graph", [False, True])
def test_batched_overlap_modes_give_the_same_bits(emix, use_graph):
    """The level-set and x-gradient positions on the second stream (every
    overlap mode) against one stream: bit for bit the same fields."""
    ws = _grids(1)
    b = emix.Batch(ws)
    out = {}
    for mode in (0, 1, 2, 3):
        b.upload()
        b.set_overlap(mode)
        b.step(3, use_graph=use_graph)
        out[mode] = [b.download(g) for g in range(len(ws))]
    for mode in (1, 2, 3):
        for g in range(len(ws)):
            assert np.array_equal(out[mode][g][0], out[0][g][0]), (mode, g, "um")
            assert np.array_equal(out[mode][g][1], out[0][g][1]), (mode, g, "phi")
    b.close()


def test_batched_grid_matches_oracle(emix, oracle):
    ws = _grids(1)
    b = emix.Batch(ws)
    b.step(1, use_graph=True)
    for g in (0, len(ws) - 1):
        w = ws[g]
        um, phi = b.download(g)
        p = oracle.step_params(w)
        d, r = oracle.inisgdm(np.ascontiguousarray(w.grid.coords()))
        rum, rphi = oracle.step(p, w.um, w.phi, w.jbn, w.mask, d, r)
        for m in range(5):
            assert_close(um[m], rum[m], what=f"grid {g} um[{m}]")
        assert_close(phi, rphi, what=f"grid {g} phi")
    b.close()


def test_autotune_keeps_results(emix):
    ws = _grids(1)
    b = emix.Batch(ws)
    ms = b.autotune(nsteps=1)
    assert ms > 0
    assert b.tuning()[1] in (32, 64, 128)
    b.step_per_grid(1)
    ref = [b.download(g) for g in range(len(ws))]
    b.upload()
    b.step(1, use_graph=True)
    for g in range(len(ws)):
        assert_close(b.download(g)[0], ref[g][0], tol=1e-13, what=f"grid {g}")
    b.close()


@pytest.mark.parametrize("steps", [2, 3, 4, 5])
def test_batched_pcr_matches_per_grid_and_oracle(emix, oracle, steps):
    """The batched step with its y/z positions by PCR + Thomas: every y/z
    position runs by PCR (the grids' pencils are at most 160 rows), the
    result agrees with the per-grid Thomas steps to rounding (1e-12) and
    with the oracle at 1e-12; a grid with longer pencils keeps Thomas."""
    ws = F.ensemble(ngrids=4, seed=13, sizes=(16, 40, 48))
    b = emix.Batch(ws)
    b.step_per_grid(2)
    ref = [b.download(g) for g in range(len(ws))]
    b.upload()
    b.set_pcr(steps)
    assert b.pcr() == steps
    assert b.pcr_positions() == 12   # per substep: gradients y, z; divergence y, z
    for use_graph in (False, True):
        b.upload()
        b.step(2, use_graph=use_graph)
        for g in range(len(ws)):
            um, phi = b.download(g)
            assert_close(um, ref[g][0], what=f"grid {g} um, {steps} PCR steps")
            assert_close(phi, ref[g][1], what=f"grid {g} phi, {steps} PCR steps")
    w = ws[0]
    p = oracle.step_params(w)
    d, r = oracle.inisgdm(np.ascontiguousarray(w.grid.coords()))
    rum, rphi = oracle.step(p, w.um, w.phi, w.jbn, w.mask, d, r, nsteps=2)
    um, phi = b.download(0)
    # per field, except the w-momentum: its largest value is the 1e-3 noise of
    # this Taylor-Green family, where one ulp of input already moves it by
    # ~2e-12 after a step (tests/test_oracle_pins.py); all five fields together
    assert_close(um, rum, what="um against the oracle")
    for m in (0, 1, 2, 4):
        assert_close(um[m], rum[m], what=f"um[{m}] against the oracle")
    assert_close(phi, rphi, what="phi against the oracle")
    b.close()
    long = F.ensemble(ngrids=2, seed=13, sizes=(16,)) + [F.random_box(16, 168, 16, seed=3, periodic=True)]
    for w in long:
        w.sgs_model = 1
    b = emix.Batch(long)
    b.set_pcr(steps)
    assert b.pcr_positions() == 6    # the y positions keep Thomas (168 rows)
    b.close()


def test_autotune_measures_pcr_depths(emix):
    ws = _grids(1)
    b = emix.Batch(ws)
    b.autotune(nsteps=1)
    ms = b.autotune_pcr_ms()
    assert sorted(ms) == [0, 2, 3, 4, 5] and all(v > 0 for v in ms.values())
    assert b.pcr() in (0, 2, 3, 4, 5)
    b.close()
