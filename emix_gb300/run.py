"""Run RK3 steps of a synthetic workload through the C ABI.

    python -m emix_gb300.run --workload tank --n 256 --steps 2 [--graph]

Used for profiling (ncu) and quick checks; prints one summary line.
"""
from __future__ import annotations

import argparse
import time


def main(argv=None):
    ap = argparse.ArgumentParser()
    ap.add_argument("--workload", default="tank", choices=["tank", "tgv"])
    ap.add_argument("--n", type=int, default=256)
    ap.add_argument("--steps", type=int, default=2)
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


if __name__ == "__main__":
    raise SystemExit(main())
