"""The FP64 gradient oracle (oracle/diff_ref.py) against FP64 central finite differences: the
reference the library's adjoint is checked against must itself be right.  CPU only."""
import numpy as np
import pytest

torch = pytest.importorskip("torch")

from oracle import diff_ref as R
from xrtailor_gb300 import scenes


def _problem(n=7, contacts=True, seed=3):
    from oracle.oracle import OracleSolver
    cloth = scenes.grid_cloth(n, 0.4, origin=(0.0, 0.0, 0.0), jitter=1e-3, seed=seed)
    pins = scenes.two_corner_pins(n)
    cloth.fixed_indices = pins
    cloth.attached_indices = pins
    p = scenes._params(num_substeps=2, num_iterations=3, stretch_compliance=1e-7,
                       bend_compliance=1e-5, enable_self_collision=0, num_collision_passes=1)
    o = OracleSolver(p)
    o.add_cloth(cloth, particle_diameter=0.02)
    o.start()
    edges, _ = o.edges()
    bends, _ = o.bends()
    prob = R.problem_from(o, p, 1e-5, colors=None)
    prob.s_colors = R.greedy_colors(edges)
    prob.b_colors = R.greedy_colors(bends)
    V = n * n
    prob.w_pinned = np.zeros(V, bool)
    prob.w_pinned[pins] = True
    if contacts:  # a plane 0.5 mm above the cloth: VF-DCD and EE-DCD records, all vertices / edges
        h = 0.0005
        pos = cloth.positions.astype(np.float64)
        plane = np.array([[[-10, h, -10], [-10, h, 10], [10, h, -10]]], np.float64)
        E = len(edges)
        ee_a = np.zeros((E, 4))
        ee_b = np.zeros((E, 4))
        ee_c = np.zeros((E, 4))
        mid = 0.5 * (pos[edges[:, 0]] + pos[edges[:, 1]])
        on = np.arange(E) % 2 == 0
        ee_a[:, 0] = np.where(on, 1e-3, 3.4e38)
        ee_a[:, 1:4] = mid + np.array([0.0, h, 0.0]) - np.array([0.003, 0.0, 0.0])
        ee_b[:, 0:3] = mid + np.array([0.0, h, 0.0]) + np.array([0.003, 0.0, 0.0])
        ee_b[:, 3] = 0.4
        ee_c[:, 0:3] = [0.0, 1.0, 0.0]
        ee_c[:, 3] = 0.6
        qs = pos.copy()
        qs[:, 1] = h
        prob.contacts = [[R.Contacts(rt_idx=-np.ones(V, np.int64), rt_qc=np.zeros((V, 3)),
                                     vf_idx=np.zeros(V, np.int64), vf_qs=qs, ee_a=ee_a,
                                     ee_b=ee_b, ee_c=ee_c, pred=plane)]]
    rng = np.random.default_rng(seed)
    E = len(edges)
    x0 = cloth.positions.astype(np.float64)
    v0 = rng.normal(0.0, 0.05, (V, 3))
    mass = rng.uniform(0.5, 2.0, V)
    comp = np.exp(rng.uniform(np.log(1e-8), np.log(1e-5), E))
    bcomp = np.full(len(bends), 1e-5)
    return prob, (x0, v0, mass, comp, bcomp)


@pytest.mark.parametrize("contacts,directions", [(False, 20), (True, 100)])
def test_reference_gradients_match_central_differences(contacts, directions):
    """7x7 mesh, one frame of 2 substeps x 3 iterations; central differences with h = 1e-6
    along random directions (relative for mass and compliance, absolute for velocity)."""
    prob, (x0, v0, mass, comp, bcomp) = _problem(contacts=contacts)
    rng = np.random.default_rng(7)
    c = rng.normal(size=x0.shape)
    g, xf = R.gradients(x0, v0, mass, comp, bcomp, prob, c)
    assert np.isfinite(xf).all()

    def L(dv, dm, dc):
        with torch.no_grad():
            x = R.rollout(*(torch.as_tensor(a, dtype=R.T) for a in
                            (x0, v0 + dv, mass + dm, comp + dc, bcomp)), prob)
        return float((x.numpy() * c).sum())

    h = 1e-6
    for k in range(directions):
        # relative perturbations of mass and compliance, absolute of velocity
        rv = rng.normal(size=v0.shape)
        rm = mass * rng.normal(size=mass.shape)
        rc = comp * rng.normal(size=comp.shape)
        fd = (L(h * rv, h * rm, h * rc) - L(-h * rv, -h * rm, -h * rc)) / (2 * h)
        ad = (g["velocity"] * rv).sum() + (g["mass"] * rm).sum() + \
            (g["stretch_compliance"] * rc).sum()
        assert abs(fd - ad) <= 1e-4 * max(abs(ad), 1e-3), (k, fd, ad)
