"""Generate the golden vectors in tests/golden/oracle_small.npz.

The reference (jramirezcr/eMix3d) ships no tests or fixtures and its Fortran
CPU path cannot be compiled here, so these vectors come from the CPU oracle
(oracle/oracle.cpp) on small seeded inputs.  They freeze the oracle: any
change to it that moves a result beyond rounding fails tests/test_golden.py.

Run from the repository root:  python tests/golden/make_golden.py
"""
from __future__ import annotations

import sys
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parents[2]
sys.path.insert(0, str(ROOT))

from emix_gb300 import fields as F  # noqa: E402
from oracle import oracle_py as O  # noqa: E402

OUT = Path(__file__).resolve().parent / "oracle_small.npz"


def stretched(nx, ny, nz):
    g = F.Grid(nx, ny, nz, (1.0, 1.2, 0.8))
    x, y, z = (g.coords1d(a) for a in range(3))
    x = x + 0.03 * np.sin(2 * np.pi * x)
    y = y ** 1.2
    z = z + 0.02 * z * z
    Z, Y, X = np.meshgrid(z, y, x, indexing="ij")
    return np.ascontiguousarray(np.stack([X, Y, Z]))


def cases():
    out = {}
    for s in (F.SCHEME_A, F.SCHEME_B, F.SCHEME_BPER, F.SCHEME_C):
        w = F.random_box(8, 7, 9, seed=100 + s, periodic=(s == F.SCHEME_BPER))
        f = np.ascontiguousarray(w.um[2])
        for ax in range(3):
            out[f"deriv_s{s}_a{ax}"] = O.deriv3d(s, ax, f, w.grid.h(ax))
    w = F.random_box(8, 7, 6, seed=7)
    vel = np.ascontiguousarray(w.um[1:4] / w.um[0])
    temp = np.ascontiguousarray(w.um[4])
    h = tuple(w.grid.h(a) for a in range(3))
    out["cudaDeriv_dvel"], out["cudaDeriv_dtemp"] = O.cudaDeriv(F.SCHEME_C, vel, temp, h)
    fl = [np.ascontiguousarray(F.uniform(8, q, w.grid.shape)) for q in range(6)]
    out["div_rs"], out["div_rsv"] = O.cuDivergence(F.SCHEME_B, *fl, np.ascontiguousarray(w.jbn), h)
    pres = np.ascontiguousarray(w.um[0] / w.mach ** 2)
    dvel = out["cudaDeriv_dvel"]
    vis = np.full(w.grid.shape, 1e-3)
    for m in range(1, 6):
        res = O.flujos(m, np.ascontiguousarray(w.um), vel, pres, dvel, np.ascontiguousarray(w.jbn), vis)
        for q, name in enumerate(("e", "f", "g", "ev", "fv", "gv")):
            out[f"flux{m}_{name}"] = res[q]
    xyz = stretched(8, 7, 6)
    out["sgs_dxyz"], out["sgs_ratios"] = O.inisgdm(xyz)
    out["sgs_sf"] = O.sgs_sf(vel, dvel, np.ascontiguousarray(w.jbn), out["sgs_dxyz"], out["sgs_ratios"])
    out["sgs_smag"] = O.sgs_smag(dvel, np.ascontiguousarray(w.jbn), out["sgs_dxyz"], 0.1)
    g = 5
    wl = F.random_box(6, 7, 8, seed=9)
    u = np.ascontiguousarray(wl.um[1:4] / wl.um[0])
    u[0] -= 0.3
    phig = O.ghost_pad(np.ascontiguousarray(wl.phi), g)
    velg = np.ascontiguousarray(np.stack([O.ghost_pad(np.ascontiguousarray(u[c]), g) for c in range(3)]))
    jbng = np.zeros((11,) + phig.shape)
    for c in (0, 4, 8):
        jbng[c] = O.ghost_pad(np.ascontiguousarray(wl.jbn[c]), g)
    hl = tuple(wl.grid.h(a) for a in range(3))
    for bugs in (0, 1):
        out[f"weno_advect_b{bugs}"] = O.weno_advect(phig, velg, np.ascontiguousarray(jbng), hl,
                                                    0.3 * min(hl), bugs)
    for kind, per, sgs in (("walls_sf", False, 2), ("periodic_smag", True, 1)):
        ws = F.random_box(8, 8, 8, seed=31, periodic=per)
        ws.sgs_model = sgs
        p = O.step_params(ws)
        d, r = O.inisgdm(np.ascontiguousarray(ws.grid.coords()))
        out[f"step_{kind}_um"], out[f"step_{kind}_phi"] = O.step(p, ws.um, ws.phi, ws.jbn,
                                                                  ws.mask, d, r)
    return out


if __name__ == "__main__":
    res = cases()
    np.savez_compressed(OUT, **res)
    print(f"wrote {OUT} ({OUT.stat().st_size} bytes, {len(res)} arrays)")
