"""The reference's checkpoint files (Fortran unformatted sequential records)
written and read by the library, cross-checked with scipy's independent
reader/writer of the same record format.  Host code only: runs without a GPU."""
import numpy as np
import pytest

from emix_gb300 import fields as F

FortranFile = pytest.importorskip("scipy.io").FortranFile


def _lib():
    from emix_gb300 import _lib
    try:
        return _lib.load()
    except OSError as e:       # library not built here
        pytest.skip(f"library not loadable: {e}")


def test_field_file_layout_matches_fortran_records(tmp_path):
    from emix_gb300 import ops
    _lib()
    w = F.random_box(7, 6, 5, seed=3)
    path = ops.write_checkpoint(str(tmp_path), 1, 7, w.um, w.mach, dto=0.125, it=42)
    assert path.endswith("field_01.007")
    f = FortranFile(path, "r", header_dtype=np.int32)
    assert f.read_ints(np.int32).tolist() == [5]
    assert f.read_ints(np.int32).tolist() == [7, 6, 5]
    u = [f.read_reals(np.float64) for _ in range(5)]
    f.close()
    r = w.um[0]
    assert np.array_equal(u[0], (w.um[1] / r).reshape(-1))
    assert np.array_equal(u[3], w.um[4].reshape(-1))
    assert np.array_equal(u[4], (r / (w.mach * w.mach)).reshape(-1))
    t = FortranFile(str(tmp_path / "time_01.007"), "r", header_dtype=np.int32)
    rec = t.read_record(np.dtype([("dto", "<f8"), ("it", "<i4")]))
    t.close()
    assert rec["dto"][0] == 0.125 and rec["it"][0] == 42
    assert ops.read_time(tmp_path / "time_01.007") == (0.125, 42)


def test_read_field_of_a_fortran_written_file(tmp_path):
    from emix_gb300 import ops
    _lib()
    nx, ny, nz = 9, 4, 6
    rng = [F.uniform(5, q, (nz, ny, nx)) for q in range(5)]
    p = tmp_path / "field_02.000"
    f = FortranFile(str(p), "w", header_dtype=np.int32)
    f.write_record(np.array([5], dtype=np.int32))
    f.write_record(np.array([nx, ny, nz], dtype=np.int32))
    for a in rng:
        f.write_record(a.astype(np.float64))
    f.close()
    um = ops.read_field(p, (nz, ny, nx), mach=0.2)
    r = rng[4] * 0.2 * 0.2
    assert np.allclose(um[0], r, rtol=0, atol=1e-15)
    assert np.array_equal(um[1], rng[0] * r)
    assert np.array_equal(um[4], rng[3])


def test_round_trip_and_checks(tmp_path):
    from emix_gb300 import ops
    lib = _lib()
    w = F.random_box(8, 7, 6, seed=4)
    path = ops.write_checkpoint(str(tmp_path), 3, 1, w.um, w.mach, 0.5, 3,
                                impellermask=np.ones(w.grid.shape))
    um = ops.read_field(path, w.grid.shape, w.mach)
    np.testing.assert_allclose(um, w.um, rtol=1e-14, atol=0)
    # leer_campos stops on a wrong number of variables or a wrong size
    with pytest.raises(ops.EmixError):
        ops.read_field(path, (6, 7, 9), w.mach)
    with pytest.raises(ops.EmixError):
        ops.read_field(path, w.grid.shape, w.mach, nd=4)
    m = np.empty(w.grid.shape)
    assert lib.emix_read_array(str(tmp_path / "impellermask_03.001").encode(), m.ctypes.data, m.size) == 0
    assert np.all(m == 1.0)


def test_sobject_file(tmp_path):
    _lib()
    from emix_gb300 import _lib as L
    nx, ny, nz = 5, 4, 3
    s = F.uniform(6, 0, (nz, ny, nx))
    p = tmp_path / "sobject.field"
    f = FortranFile(str(p), "w", header_dtype=np.int32)
    f.write_record(np.array([nx, ny, nz], dtype=np.int32))
    f.write_record(s)
    f.close()
    out = np.empty_like(s)
    assert L.load().emix_read_sobject(str(p).encode(), nx, ny, nz, out.ctypes.data) == 0
    assert np.array_equal(out, s)
