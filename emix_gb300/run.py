"""Run RK3 steps of a synthetic workload through the C ABI.

    python -m emix_gb300.run --workload tank --n 256 --steps 2 [--graph]
    python -m emix_gb300.run --operators --n 192
    python -m emix_gb300.run --workload ensemble --steps 2

Used for profiling (ncu) and quick checks; prints one summary line.
--operators runs every standalone device operator of the library once (after
one warm-up pass) on the n^3 tank's fields, so that a launch list of it covers
the kernels outside the RK3 step.
"""
from __future__ import annotations

import argparse
import time


def main(argv=None):
    ap = argparse.ArgumentParser()
    ap.add_argument("--workload", default="tank", choices=["tank", "tgv", "ensemble"])
    ap.add_argument("--operators", action="store_true",
                    help="run each standalone device operator once (after a warm-up pass)")
    ap.add_argument("--n", type=int, default=256)
    ap.add_argument("--steps", type=int, default=2)
    ap.add_argument("--grids", type=int, default=48, help="ensemble: the first N grids of the 48-grid draw")
    ap.add_argument("--graph", action="store_true")
    ap.add_argument("--no-level-set", action="store_true")
    ap.add_argument("--walls", action="store_true", help="frontera wall conditions every substep")
    ap.add_argument("--impeller", action="store_true", help="rotating impeller forcing (tank)")
    ap.add_argument("--adjoint", action="store_true",
                    help="forward + reverse sweep of the tank objective (implies --impeller --walls)")
    a = ap.parse_args(argv)
    import numpy as np
    import torch
    from . import fields as F
    from . import ops
    if a.operators:
        operators(a.n)
        return 0
    if a.workload == "ensemble":
        b = ops.Batch(F.ensemble(ngrids=a.grids, seed=7))
        b.upload()
        t0 = time.perf_counter()
        b.step(a.steps, use_graph=a.graph)
        torch.cuda.synchronize()
        sec = time.perf_counter() - t0
        um = b.download(0)[0]
        ok = bool(np.isfinite(um).all())
        print(f"ensemble of {a.grids} grids ({b.ncell} cells): {a.steps} batched steps in {sec:.3f} s, "
              f"finite={ok}")
        b.close()
        return 0 if ok else 1
    if a.adjoint:
        w = F.stirred_tank(n=a.n, impeller=True)
        r = ops.TankGradient(w, a.steps, 1, bc_walls=1)
        t0 = time.perf_counter()
        J = r.run(w.impeller.omega, w.cs)
        g = r.adj.backward()
        torch.cuda.synchronize()
        print(f"{w.name}: J={J:.12g} dJ/domega={g[0]:.6g} dJ/dCs={g[1]:.6g} "
              f"in {time.perf_counter() - t0:.3f} s")
        r.close()
        return 0
    w = F.stirred_tank(n=a.n, impeller=a.impeller) if a.workload == "tank" else F.taylor_green(n=a.n)
    ctx = ops.Context(w, level_set=not a.no_level_set, bc_walls=int(a.walls))
    t0 = time.perf_counter()
    ctx.step(a.steps, use_graph=a.graph)
    torch.cuda.synchronize()
    sec = time.perf_counter() - t0
    um, phi = ctx.download()
    ok = bool(np.isfinite(um).all() and (phi is None or np.isfinite(phi).all()))
    print(f"{w.name}: {a.steps} steps in {sec:.3f} s, finite={ok}, max|um|={float(np.abs(um).max()):.6g}")
    ctx.close()
    return 0 if ok else 1


def operators(n: int, passes: int = 2) -> None:
    """Each device operator once per pass on the n^3 tank's fields."""
    import numpy as np
    import torch
    from . import fields as F
    from . import ops
    w = F.stirred_tank(n=n, impeller=True)
    dev = lambda a: torch.from_numpy(np.ascontiguousarray(a)).cuda()
    g = 5
    hs = tuple(w.grid.h(a) for a in range(3))
    xyz = dev(w.grid.coords())
    jbn = dev(w.jbn)
    um = dev(w.um)
    r = um[0]
    u = torch.stack([um[1] / r, um[2] / r, um[3] / r]).contiguous()
    pres = r / w.mach ** 2
    phi = dev(w.phi)
    sobj = 0.3 - torch.sqrt(xyz[0] ** 2 + xyz[1] ** 2 + (xyz[2] - 0.7) ** 2)
    nxg = n + 2 * g
    phig = ops.ghost_pad_dev(phi, g)
    velg = torch.stack([ops.ghost_pad_dev(u[d].contiguous(), g) for d in range(3)]).contiguous()
    jbng = torch.stack([ops.ghost_pad_dev(jbn[c].contiguous(), g) for c in range(11)]).contiguous()
    dmins = torch.full_like(phig, min(hs))
    # the PCR form takes pencils of at most 160 rows: y and z cut to 160
    m = min(n, 160)
    us = u[:, :m, :m, :].contiguous()
    for _ in range(passes):
        ops.deriv_dev(u, 0, hs[0], F.SCHEME_B)
        ops.deriv_pcr_dev(us, 1, hs[1], 3, F.SCHEME_B)
        ops.deriv_t_dev(u, 1, hs[1], F.SCHEME_B)
        dvel, dtemp = ops.cudaDeriv_dev(u, um[4].contiguous(), hs, F.SCHEME_C)
        dxyz, ratios = ops.sgs_setup_dev(xyz)
        amut, vis = ops.sgs_viscosity_dev(2, 0.1781, 1e-3, u, dvel, jbn, dxyz, ratios)
        fl = ops.flux_dev(2, um, u, pres, dvel, jbn, vis)
        ops.cuDivergence_dev(*fl, jbn, hs, F.SCHEME_C)
        ops.weno5_advect_dev(phig.clone(), velg, jbng, hs, 0.5 * min(hs))
        ops.reinit_dev(phig.clone(), jbng, dmins, hs, g, min(hs), iters=2)
        ops.filtrado_dev(um.clone(), jbn, 0.49)
        ops.advect_extrapolate_dev(pres.clone(), jbn, sobj.contiguous(), hs, 0.8 * min(hs))
        ops.impeller_force_dev(um.clone(), xyz, w.impeller, 0.1)
        ops.bc_walls_dev(um.clone())
        ops.cfl_dev(u, xyz, w.mach)
        ops.metrics_dev(xyz, hs)
        ops.ghost_unpad_dev(phig, g)
    torch.cuda.synchronize()
    print(f"operators on {n}^3 ({nxg}^3 padded): {passes} passes, ok")


if __name__ == "__main__":
    raise SystemExit(main())
