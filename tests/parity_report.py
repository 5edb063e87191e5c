"""Per-output parity of the CUDA library: the normwise relative L-inf error of
every output against the CPU oracle (and, for the operators the reference
also has in CUDA, against the reference kernels' own recorded outputs in
tests/golden/reference_cuda.npz).  The tests assert the bar (1e-12; for the
Taylor-Green w-momentum, twice the oracle's own spread under one ulp of input
perturbation); this prints the errors themselves as a markdown table.  Needs
a GPU:

    python tests/parity_report.py
"""
from __future__ import annotations

import importlib.util
import sys
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
sys.path.insert(0, str(HERE.parent))
sys.path.insert(0, str(HERE))

from emix_gb300 import fields as F   # noqa: E402
from helpers import relerr           # noqa: E402

ROWS: list[tuple[str, str, float]] = []


def row(what: str, against: str, err: float) -> None:
    ROWS.append((what, against, err))


def main() -> int:
    import torch
    from emix_gb300 import ops as E
    from oracle import oracle_py as O
    O.load()

    def dev(a):
        return torch.from_numpy(np.ascontiguousarray(a)).cuda()

    def host(t):
        torch.cuda.synchronize()
        return t.cpu().numpy()

    names = {F.SCHEME_A: "A", F.SCHEME_B: "B", F.SCHEME_BPER: "B cyclic", F.SCHEME_C: "C"}
    # compact first derivative, every scheme and axis
    for sch in (F.SCHEME_A, F.SCHEME_B, F.SCHEME_BPER, F.SCHEME_C):
        w = F.random_box(24, 20, 28, seed=11, periodic=(sch == F.SCHEME_BPER))
        f = np.ascontiguousarray(w.um[1:4])
        for ax in range(3):
            h = w.grid.h(ax)
            got = host(E.deriv_dev(dev(f), ax, h, sch))
            e = max(relerr(got[c], O.deriv3d(sch, ax, f[c], h)) for c in range(3))
            row(f"D, scheme {names[sch]}, axis {'xyz'[ax]} (24x20x28, 3 fields)", "oracle", e)
    # cudaDeriv (host form), cuDivergence
    w = F.random_box(20, 18, 22, seed=3)
    vel = np.ascontiguousarray(w.um[1:4] / w.um[0])
    temp = np.ascontiguousarray(w.um[4])
    h = tuple(w.grid.h(a) for a in range(3))
    dv, dt_ = E.cudaDeriv(vel, temp, h, F.SCHEME_C)
    rdv, rdt = O.cudaDeriv(F.SCHEME_C, vel, temp, h)
    row("cudaDeriv dVel (9 outputs, max)", "oracle", max(relerr(dv[c], rdv[c]) for c in range(9)))
    row("cudaDeriv dTemp (3 outputs, max)", "oracle", max(relerr(dt_[c], rdt[c]) for c in range(3)))
    w = F.random_box(18, 16, 20, seed=7)
    fl = [np.ascontiguousarray(F.uniform(21, q, w.grid.shape)) for q in range(6)]
    jbn = np.ascontiguousarray(w.jbn)
    h = tuple(w.grid.h(a) for a in range(3))
    rs, rsv = E.cuDivergence(*fl, jbn, h, F.SCHEME_C)
    r_rs, r_rsv = O.cuDivergence(F.SCHEME_C, *fl, jbn, h)
    row("cuDivergence rs", "oracle", relerr(rs, r_rs))
    row("cuDivergence rsv", "oracle", relerr(rsv, r_rsv))
    # fluxes, SGS
    w = F.random_box(14, 12, 10, seed=9)
    n = w.grid.shape
    um = np.ascontiguousarray(w.um)
    u = np.ascontiguousarray(w.um[1:4] / w.um[0])
    pres = np.ascontiguousarray(w.um[0] / w.mach ** 2)
    dvel = np.ascontiguousarray(np.stack([F.uniform(31, q, n) for q in range(9)]))
    vis = np.ascontiguousarray(1e-3 + 1e-4 * (1 + F.uniform(32, 0, n)))
    for neq in range(1, 6):
        got = E.flux_dev(neq, dev(um), dev(u), dev(pres), dev(dvel), dev(jbn := np.ascontiguousarray(w.jbn)), dev(vis))
        ref = O.flujos(neq, um, u, pres, dvel, jbn, vis)
        row(f"flujos equation {neq} (6 fluxes, max)", "oracle", max(relerr(host(got[q]), ref[q]) for q in range(6)))
    w = F.random_box(16, 14, 12, seed=12)
    g = F.Grid(16, 14, 12, (1.0, 1.2, 0.8))
    x, y, z = (g.coords1d(a) for a in range(3))
    Z, Y, X = np.meshgrid(z + 0.02 * z * z, y ** 1.2, x + 0.03 * np.sin(2 * np.pi * x), indexing="ij")
    xyz = np.ascontiguousarray(np.stack([X, Y, Z]))
    dxyz, ratios = O.inisgdm(xyz)
    d_, r_ = E.sgs_setup_dev(dev(xyz))
    row("INISGDM filter width", "oracle", relerr(host(d_), dxyz))
    u = np.ascontiguousarray(w.um[1:4] / w.um[0])
    h = tuple(w.grid.h(a) for a in range(3))
    dvel, _ = O.cudaDeriv(F.SCHEME_B, u, np.ascontiguousarray(w.um[4]), h)
    jbn = np.ascontiguousarray(w.jbn)
    amut, _ = E.sgs_viscosity_dev(1, 0.1, 1e-3, dev(u), dev(dvel), dev(jbn), dev(dxyz))
    row("Smagorinsky amut", "oracle", relerr(host(amut), O.sgs_smag(dvel, jbn, dxyz, 0.1)))
    amut, _ = E.sgs_viscosity_dev(2, 0.1781, 1e-3, dev(u), dev(dvel), dev(jbn), dev(dxyz), dev(ratios))
    row("structure-function amut", "oracle", relerr(host(amut), O.sgs_sf(u, dvel, jbn, dxyz, ratios, 0.1781)))
    # full steps
    cases = {
        "periodic box, Smagorinsky (16x18x14)": (F.random_box(16, 18, 14, seed=21, periodic=True), 1, 2),
        "walls, structure function (14x16x18)": (F.random_box(14, 16, 18, seed=22, periodic=False), 2, 2),
        "walls, scheme C (16x14x16)": (F.random_box(16, 14, 16, seed=23, periodic=False, scheme=F.SCHEME_C), 1, 2),
        "Taylor-Green 64^3 periodic": (F.taylor_green(64), 1, 10),
    }
    for name, (w, sgs, nsteps) in cases.items():
        w.sgs_model = sgs
        ctx = E.Context(w, level_set=True)
        ctx.step(nsteps, use_graph=True)
        got_um, got_phi = ctx.download()
        ctx.close()
        p = O.step_params(w, level_set=True)
        dx, rt = O.inisgdm(np.ascontiguousarray(w.grid.coords()))
        rum, rphi = O.step(p, w.um, w.phi, w.jbn, w.mask, dx, rt, nsteps=nsteps)
        e = max(relerr(got_um[m], rum[m]) for m in range(5))
        row(f"step x{nsteps}, {name}: um (5 fields, max)", "oracle", e)
        row(f"step x{nsteps}, {name}: phi", "oracle", relerr(got_phi, rphi))
    w = F.stirred_tank(n=24, impeller=True, impeller_omega=1.3)
    ctx = E.Context(w, bc_walls=1)
    ctx.step(3)
    got_um, got_phi = ctx.download()
    ctx.close()
    p = O.step_params(w, bc_walls=1)
    dx, rt = O.inisgdm(np.ascontiguousarray(w.grid.coords()))
    rum, rphi = O.step(p, w.um, w.phi, w.jbn, w.mask, dx, rt, nsteps=3)
    row("step x3, tank 24^3 walls + impeller: um (5 fields, max)", "oracle",
        max(relerr(got_um[m], rum[m]) for m in range(5)))
    row("step x3, tank 24^3 walls + impeller: phi", "oracle", relerr(got_phi, rphi))
    # the Taylor-Green box per field, beside the oracle's own spread when its
    # inputs move by one ulp (seeded directions)
    w = F.taylor_green(64)
    ctx = E.Context(w, level_set=True)
    ctx.step(10, use_graph=True)
    got_um, got_phi = ctx.download()
    ctx.close()
    p = O.step_params(w, level_set=True)
    dx, rt = O.inisgdm(np.ascontiguousarray(w.grid.coords()))
    rum, rphi = O.step(p, w.um, w.phi, w.jbn, w.mask, dx, rt, nsteps=10)

    def nudged(x, seed):
        d = np.random.default_rng(seed).integers(0, 2, size=x.shape).astype(bool)
        return np.where(d, np.nextafter(x, np.inf), np.nextafter(x, -np.inf))

    sum_, _ = O.step(p, nudged(w.um, 5), nudged(w.phi, 6), w.jbn, w.mask, dx, rt, nsteps=10)
    for m in range(5):
        row(f"step x10, Taylor-Green 64^3: um[{m}]", "oracle", relerr(got_um[m], rum[m]))
        row(f"step x10, Taylor-Green 64^3: um[{m}]", "oracle with inputs moved by one ulp", relerr(sum_[m], rum[m]))
    # the benchmark's own sizes: the 256^3 tank one step through the host-buffer
    # entry point, the 128^3 tank 8 steps through the device context
    for n, nsteps in ((256, 1), (128, 8)):
        w = F.stirred_tank(n=n, impeller=True)
        ctx = E.Context(w, level_set=True, ls_ghost=5, bc_walls=1)
        if nsteps == 1:
            got_um = np.ascontiguousarray(w.um.copy())
            got_phi = np.ascontiguousarray(w.phi.copy())
            ctx.step_host(got_um, got_phi, 1)
        else:
            ctx.step(nsteps, use_graph=True)
            got_um, got_phi = ctx.download()
        ctx.close()
        p = O.step_params(w, level_set=True, bc_walls=1)
        dx, rt = O.inisgdm(np.ascontiguousarray(w.grid.coords()))
        rum, rphi = O.step(p, w.um, w.phi, w.jbn, w.mask, dx, rt, nsteps=nsteps)
        for m in range(5):
            row(f"step x{nsteps}, tank {n}^3 walls + impeller: um[{m}]", "oracle", relerr(got_um[m], rum[m]))
        row(f"step x{nsteps}, tank {n}^3 walls + impeller: phi", "oracle", relerr(got_phi, rphi))
    # the y/z derivative by PCR + Thomas
    w = F.random_box(24, 48, 40, seed=31)
    f = np.ascontiguousarray(w.um[1:4])
    for steps in (2, 3, 4, 5):
        got = host(E.deriv_pcr_dev(dev(f), 1, w.grid.h(1), steps, F.SCHEME_B))
        e = max(relerr(got[c], O.deriv3d(F.SCHEME_B, 1, f[c], w.grid.h(1))) for c in range(3))
        row(f"D by PCR ({steps} steps) + Thomas, scheme B, axis y (24x48x40, 3 fields)", "oracle", e)
    # against the reference's own CUDA kernels
    gold_path = HERE / "golden" / "reference_cuda.npz"
    spec = importlib.util.spec_from_file_location("mg", HERE / "golden" / "make_reference_golden.py")
    mg = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(mg)
    gold = dict(np.load(gold_path))
    for name, f in mg.deriv_cases():
        for ax in range(3):
            hh = float(gold[f"{name}_h{ax}"])
            got = host(E.deriv_dev(dev(f), ax, hh, F.SCHEME_C))
            row(f"D scheme C, {name} axis {'xyz'[ax]}", "reference cu::cs::dF kernels", relerr(got, gold[f"{name}_a{ax}"]))
    fl, jb = mg.div_case()
    rs, rsv = E.cuDivergence(*[np.ascontiguousarray(a) for a in fl], np.ascontiguousarray(jb), tuple(gold["div_h"]), F.SCHEME_C)
    row("cuDivergence rs", "reference cuDivergence", relerr(rs, gold["div_rs"]))
    row("cuDivergence rsv", "reference cuDivergence", relerr(rsv, gold["div_rsv"]))
    wp, wv, wj, _, _ = mg.weno_case()
    out = E.weno5_advect(np.ascontiguousarray(wp), np.ascontiguousarray(wv), np.ascontiguousarray(wj),
                         tuple(gold["weno_h"]), float(gold["weno_dt"]), 1)
    row("WENO5 TVD-RK3 step (cuAdvectLsJB)", "reference lsTools/extrapol kernels", relerr(out, gold["weno_out"]))
    if "extrap_out" in gold:
        pr, ej, es, ed, em = mg.extrap_case()
        out = E.advect_extrapolate(pr, ej, es, ed, em)
        row("advect_CUDA pressure extrapolation", "reference advect_CUDA", relerr(out, gold["extrap_out"]))
    if "reinit_out" in gold:
        rp, rj, rd, rh, rdm, ri = mg.reinit_case()
        t = dev(rp.copy())
        E.reinit_dev(t, dev(rj), dev(rd), rh, 5, rdm, iters=ri, ref_bugs=1)
        row("reinitialisation (cuReinitLsJB)", "reference kernels", relerr(host(t), gold["reinit_out"]))

    print("| output | against | normwise relative L-inf error |")
    print("|---|---|---|")
    for what, against, e in ROWS:
        print(f"| {what} | {against} | {e:.2e} |")
    return 0


if __name__ == "__main__":
    sys.exit(main())
