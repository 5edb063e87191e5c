"""The fused launches (the gradients' y and z passes as one launch, the
Smagorinsky viscosity with the fluxes) against every operator in a launch of
its own (emix_ctx_set_fusion(0)): the same values bit for bit, in the
graph-replayed step, the eager step, and the adjoint's taped forward (its
reverse sweep to rounding: it sums with atomics)."""
import numpy as np
import pytest

from emix_gb300 import fields as F

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("use_graph", [True, False])
def test_fused_step_equals_separate_launches(use_graph):
    from emix_gb300 import ops
    w = F.stirred_tank(n=24, impeller=True, impeller_omega=1.3)
    out = []
    for fuse in (True, False):
        ctx = ops.Context(w, bc_walls=1)
        ctx.set_fusion(fuse)
        ctx.step(3, use_graph=use_graph)
        out.append(ctx.download())
        # the tank's plan: 36 records, 3 of each fused pair per step
        assert ctx.launches_per_step() == (30 if fuse else 36)
        ctx.close()
    (u0, p0), (u1, p1) = out
    assert np.array_equal(u0, u1) and np.array_equal(p0, p1)


def test_fused_taped_forward_equals_separate_launches():
    from emix_gb300 import ops
    w = F.stirred_tank(n=24, impeller=True, impeller_omega=1.3)
    res = []
    for fuse in (True, False):
        r = ops.TankGradient(w, 2, 0, bc_walls=1)
        r.ctx.set_fusion(fuse)
        J = r.run(1.3, 0.1)
        g = r.adj.backward()
        um, phi = r.ctx.download()
        res.append((J, g, um, phi))
        r.close()
    (J0, g0, u0, f0), (J1, g1, u1, f1) = res
    # the forward (tapes, final state, J) is bitwise the same; the reverse
    # sweep scatters with atomics, so its sums may round in another order
    assert J0 == J1
    assert np.array_equal(u0, u1) and np.array_equal(f0, f1)
    for a, b in zip(g0, g1):
        assert abs(a - b) <= 1e-14 * abs(b), (a, b)

