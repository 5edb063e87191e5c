"""Run the reference's own CUDA kernels on seeded inputs and save their outputs
as golden vectors (tests/golden/reference_cuda.npz).

The reference's Fortran CPU path cannot be compiled here, but its CUDA kernels
can: oracle/ref/build_ref.sh compiles src/Schemes/derivCompact.cu (via
solver/cuDeriv.cu), solver/cuDivergence.cu, src/LevelSet/lsTools.cu and
src/LevelSet/extrapol.cu, unmodified, into cubins under oracle/_ref/ (on the
build host, where the sources are).  This script builds the harness
oracle/ref/ref_harness.cu and runs those kernels on a GPU, so it runs on the
GPU machine:

    python tests/golden/make_reference_golden.py [out.npz]

Cases: the variant-C compact derivative along each axis (cu::cs::dFdX/Y/Z),
cuDivergence, one cuAdvectLsJB WENO5 TVD-RK3 step, the ghost padding of
advect_CUDA, and advect_CUDA itself (the pressure extrapolation into the
solid) and cuReinitLsJB (level-set reinitialisation).  Only the reference's
outputs are stored; the inputs are regenerated from seeds by deriv_cases(),
div_case(), weno_case(), pad_case(), extrap_case() and reinit_case() below.
"""
from __future__ import annotations

import os
import subprocess
import sys
import tempfile
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parents[2]
sys.path.insert(0, str(ROOT))

from emix_gb300 import fields as F  # noqa: E402

HARNESS_SRC = ROOT / "oracle" / "ref" / "ref_harness.cu"
REF_DIR = ROOT / "oracle" / "_ref"
HARNESS = ROOT / "oracle" / "_build" / "ref_harness"


def build_harness():
    HARNESS.parent.mkdir(exist_ok=True)
    subprocess.run(["nvcc", "-O2", "-std=c++17", f"-I{REF_DIR}", "-o", str(HARNESS), str(HARNESS_SRC),
                    "-lcuda"], check=True)


def run(*args):
    p = subprocess.run([str(HARNESS), *map(str, args)], capture_output=True, text=True,
                       env={**os.environ, "EMIX_REF_DIR": str(REF_DIR)})
    if p.returncode != 0:
        raise RuntimeError(f"harness {args[0]} failed: {p.stdout}\n{p.stderr}")


def deriv_cases():
    """(name, field, h) -- shapes (nx, ny, nz) with C-order arrays (nz, ny, nx)."""
    out = []
    for q, (nx, ny, nz) in enumerate([(24, 20, 28), (40, 12, 7)]):
        f = np.ascontiguousarray(F.uniform(61, q, (nz, ny, nx)) + np.sin(np.arange(nx) / 3.0))
        out.append((f"deriv{q}", f))
    return out


def div_case():
    nx, ny, nz = 20, 18, 22
    fl = [np.ascontiguousarray(F.uniform(62, q, (nz, ny, nx))) for q in range(6)]
    jbn = np.zeros((11, nz, ny, nx))
    for c in range(11):
        jbn[c] = 0.5 + 0.25 * (F.uniform(63, c, (nz, ny, nx)) + 1.0)
    return fl, np.ascontiguousarray(jbn)


def weno_case():
    nxg, nyg, nzg = 30, 30, 25
    sh = (nzg, nyg, nxg)
    z, y, x = np.meshgrid(np.arange(nzg) / nzg, np.arange(nyg) / nyg, np.arange(nxg) / nxg,
                          indexing="ij")
    phi = np.sqrt((x - 0.45) ** 2 + (y - 0.55) ** 2 + (z - 0.5) ** 2) - 0.3 + 0.01 * F.uniform(64, 0, sh)
    vel = np.stack([0.6 * np.sin(2 * np.pi * y) - 0.1, -0.5 * np.sin(2 * np.pi * x),
                    0.3 * np.cos(2 * np.pi * x) + 0.05 * F.uniform(64, 1, sh)])
    jbn = np.zeros((11,) + sh)
    for c in (0, 4, 8):
        jbn[c] = 1.0 + 0.1 * F.uniform(64, 2 + c, sh)
    h = (1.0 / 20, 1.0 / 20, 1.0 / 15)
    return np.ascontiguousarray(phi), np.ascontiguousarray(vel), np.ascontiguousarray(jbn), h, 0.01


def pad_case():
    return np.ascontiguousarray(F.uniform(65, 0, (20, 20, 20)))


def extrap_case():
    """press, jbn (11), sobject (a sphere, > 0 inside the solid), delta, deltamin."""
    n = 20
    sh = (n, n, n)
    z, y, x = np.meshgrid(*(np.arange(n) / (n - 1),) * 3, indexing="ij")
    sobj = 0.32 - np.sqrt((x - 0.45) ** 2 + (y - 0.55) ** 2 + (z - 0.5) ** 2)
    press = np.sin(3 * x) + np.cos(2 * y) * z + 0.01 * F.uniform(66, 0, sh)
    jbn = np.zeros((11,) + sh)
    for c in range(11):
        jbn[c] = F.uniform(66, 1 + c, sh)
    for c in (0, 4, 8):
        jbn[c] = 1.0 + 0.1 * F.uniform(66, 20 + c, sh)
    return (np.ascontiguousarray(press), np.ascontiguousarray(jbn), np.ascontiguousarray(sobj),
            (0.05, 0.055, 0.06), 0.04)


def reinit_case():
    """Padded 30^3 level set (a distorted sphere distance), padded metric,
    smoothing widths, spacings, deltamin, iterations."""
    n = 30
    z, y, x = np.meshgrid(*(np.arange(n) / (n - 1),) * 3, indexing="ij")
    d = np.sqrt((x - 0.5) ** 2 + (y - 0.45) ** 2 + (z - 0.55) ** 2) - 0.25
    phi = 2.5 * d * (1.0 + 0.3 * np.sin(5 * x)) + 1e-3 * F.uniform(67, 0, d.shape)
    jbn = np.zeros((11,) + d.shape)
    for c in range(11):
        jbn[c] = F.uniform(67, 1 + c, d.shape)
    for c in (0, 4, 8):
        jbn[c] = 1.0 + 0.05 * F.uniform(67, 20 + c, d.shape)
    h = (1.0 / 29, 1.0 / 29, 1.0 / 29)
    dm = np.full(d.shape, 0.8 / 29)
    return (np.ascontiguousarray(phi), np.ascontiguousarray(jbn), np.ascontiguousarray(dm), h,
            0.8 / 29, 10)


def main(out_path=None):
    out_path = Path(out_path) if out_path else Path(__file__).resolve().parent / "reference_cuda.npz"
    build_harness()
    res = {}
    with tempfile.TemporaryDirectory() as td:
        td = Path(td)

        def wr(name, a):
            p = td / f"{name}.bin"
            np.ascontiguousarray(a, dtype=np.float64).tofile(p)
            return p

        for name, f in deriv_cases():
            nz, ny, nx = f.shape
            for axis in range(3):
                n = (nx, ny, nz)[axis]
                h = 1.0 / (n - 1)
                o = td / "o.bin"
                run("deriv", nx, ny, nz, axis, repr(h), wr("f", f), o)
                res[f"{name}_a{axis}"] = np.fromfile(o).reshape(f.shape)
                res[f"{name}_h{axis}"] = np.array(h)
        fl, jbn = div_case()
        nz, ny, nx = fl[0].shape
        hs = (1.0 / (nx - 1), 1.0 / (ny - 1), 1.0 / (nz - 1))
        paths = [wr(f"fl{q}", a) for q, a in enumerate(fl)]
        run("div", nx, ny, nz, *map(repr, hs), *paths, wr("jbn", jbn), td / "rs.bin", td / "rsv.bin")
        res["div_h"] = np.array(hs)
        res["div_rs"] = np.fromfile(td / "rs.bin").reshape(fl[0].shape)
        res["div_rsv"] = np.fromfile(td / "rsv.bin").reshape(fl[0].shape)
        phi, vel, jw, h, dt = weno_case()
        nzg, nyg, nxg = phi.shape
        run("weno", nxg, nyg, nzg, *map(repr, h), repr(dt), wr("phi", phi), wr("vel", vel),
            wr("jw", jw), td / "phi_out.bin")
        res.update(weno_h=np.array(h), weno_dt=np.array(dt),
                   weno_out=np.fromfile(td / "phi_out.bin").reshape(phi.shape))
        val = pad_case()
        run("pad", 20, 20, 20, 5, wr("val", val), td / "pad.bin")
        res.update(pad_out=np.fromfile(td / "pad.bin").reshape(30, 30, 30))
        press, jbn, sobj, delta, dmin = extrap_case()
        run("extrap", 20, 20, 20, *map(repr, delta), repr(dmin), wr("press", press), wr("jbn", jbn),
            wr("sobj", sobj), td / "extrap.bin")
        res.update(extrap_out=np.fromfile(td / "extrap.bin").reshape(press.shape))
        phi, jbn, dm, h, dmin, iters = reinit_case()
        run("reinit", 30, 30, 30, 5, *map(repr, h), repr(dmin), iters, wr("rphi", phi),
            wr("rjbn", jbn), wr("rdm", dm), td / "reinit.bin")
        res.update(reinit_out=np.fromfile(td / "reinit.bin").reshape(phi.shape))
    np.savez_compressed(out_path, **res)
    print(f"wrote {out_path} ({out_path.stat().st_size} bytes, {len(res)} arrays)")


if __name__ == "__main__":
    main(sys.argv[1] if len(sys.argv) > 1 else None)
