"""emix_step_host, the host-buffer entry point (the one the end-to-end figure
times): the same values as the device-resident steps, bit for bit.  Its first
step uploads phi, then um by z-slabs on a second stream, and runs the
primitive variables and the first level-set stage on each slab as it lands;
its last step moves the last
level-set stage after the last RK update, copies um back by z-slabs of that
update and phi by z-slabs of the stage.  The cases below cover one, two and
three steps, walls and the periodic box, uneven and shallow z extents (fewer
upload slabs), the context's steps on one stream and with the level-set
stages alone on the second, the forms that copy plainly instead (the
impeller's blade-edge interpolation after the RK update, no level set), a
filter step last (uploads overlapped, copies after the filter) and pageable
host buffers."""
import numpy as np
import pytest

from emix_gb300 import fields as F

pytestmark = pytest.mark.gpu


def _tank(interp=0):
    w = F.stirred_tank(n=24, impeller=True, impeller_omega=1.3)
    w.impeller.interp = interp
    return w


def _device(w, nsteps, **kw):
    from emix_gb300 import ops
    ctx = ops.Context(w, **kw)
    ctx.step(nsteps, use_graph=True)
    um, phi = ctx.download()
    idx = ctx.step_index
    ctx.close()
    return um, phi, idx


def _host(w, nsteps, pinned=True, overlap=None, level_set=True, **kw):
    import torch
    from emix_gb300 import ops
    ctx = ops.Context(w, level_set=level_set, **kw)
    if overlap is not None:
        ctx.set_overlap(overlap)
    um_t = torch.from_numpy(np.ascontiguousarray(w.um))
    phi_t = torch.from_numpy(np.ascontiguousarray(w.phi))
    if pinned:
        um_t, phi_t = um_t.pin_memory(), phi_t.pin_memory()
    else:
        um_t, phi_t = um_t.clone(), phi_t.clone()
    um, phi = um_t.numpy(), phi_t.numpy()
    ctx.step_host(um, phi if level_set else None, nsteps)
    idx = ctx.step_index
    ctx.close()
    return um.copy(), (phi.copy() if level_set else None), idx


@pytest.mark.parametrize("nsteps", [1, 2, 3])
@pytest.mark.parametrize("pinned", [True, False])
def test_step_host_matches_device_steps(nsteps, pinned):
    w = _tank()
    um, phi, idx = _device(w, nsteps, bc_walls=1)
    hum, hphi, hidx = _host(w, nsteps, pinned=pinned, bc_walls=1)
    assert hidx == idx == nsteps
    assert np.array_equal(hum, um)
    assert np.array_equal(hphi, phi)


@pytest.mark.parametrize("case", ["nz23", "nz9", "nz14", "periodic", "static_mask"])
def test_step_host_shapes(case):
    """Uneven slab cuts (nz = 23), a single upload slab (nz = 9 with 5 ghost
    layers), two (nz = 14), the periodic box without walls and the tank
    without the rotating impeller."""
    kw = {"bc_walls": 1}
    if case == "periodic":
        w = F.taylor_green(20)
        kw = {}
    elif case == "static_mask":
        w = F.stirred_tank(n=20, nz=18)
    else:
        w = F.stirred_tank(n=18, nz=int(case[2:]), impeller=True, impeller_omega=1.3)
    for nsteps in (1, 2):
        um, phi, idx = _device(w, nsteps, **kw)
        hum, hphi, hidx = _host(w, nsteps, **kw)
        assert hidx == idx == nsteps
        assert np.array_equal(hum, um), f"{case}, {nsteps} steps: um"
        assert np.array_equal(hphi, phi), f"{case}, {nsteps} steps: phi"


@pytest.mark.parametrize("case", ["one_stream", "stages_only", "filter_last", "interp", "no_level_set"])
def test_step_host_forms(case):
    kw = {"bc_walls": 1}
    w = _tank(interp=1 if case == "interp" else 0)
    nsteps = 3 if case == "filter_last" else 2
    if case == "filter_last":
        # one step whose filter is due: uploads overlapped, copies after the filter
        kw1 = dict(kw, filter_every=1, cfilt=0.2)
        um, phi, idx = _device(w, 1, **kw1)
        hum, hphi, hidx = _host(w, 1, **kw1)
        assert hidx == idx == 1
        assert np.array_equal(hum, um) and np.array_equal(hphi, phi)
    if case == "filter_last":
        kw.update(filter_every=2, cfilt=0.2)   # steps 0 and 2 filter: the last one does
    ls = case != "no_level_set"
    um, phi, idx = _device(w, nsteps, level_set=ls, **kw)
    ov = {"one_stream": 0, "stages_only": 1}.get(case)
    hum, hphi, hidx = _host(w, nsteps, overlap=ov, level_set=ls, **kw)
    assert hidx == idx == nsteps
    assert np.array_equal(hum, um)
    if ls:
        assert np.array_equal(hphi, phi)


def test_step_host_zero_steps_returns_the_inputs():
    w = _tank()
    hum, hphi, idx = _host(w, 0, bc_walls=1)
    assert idx == 0
    assert np.array_equal(hum, w.um) and np.array_equal(hphi, w.phi)
