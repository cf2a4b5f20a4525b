"""Hand-written adjoint (include/xrt_diff.h) against the FP64 reference autodiff
(oracle/diff_ref.py, itself checked against central finite differences): gradients with respect
to per-edge stretch compliance, per-bend compliance, per-vertex mass, initial velocity and
initial position, through stretch, bend, LRA, obstacle contacts held as recorded, predict and
finalize.

Tolerances.  The library computes in float32, so its gradients carry the float32 error floor of
the reference's own formulas.  Each test evaluates the same reference program under
`diff_ref.precision(torch.float32)` and bounds the library's relative error by a small multiple
of that program's error (plus a floor).  Where the frame is well conditioned in float32 (no
bending), the library's gradients must also match the float32 autodiff of the same program to
1e-4: that isolates the hand-written adjoint from the forward's rounding (measured: 1e-7 to
6e-6).  The reference's bend constraint is the stiff, badly
conditioned part in single precision: its rest angle takes the second normal with the opposite
orientation to the solve (BasicSolverHelper.cu:8-72 against the rest-angle setup), so a flat
sheet starts a quarter turn from its target and folds; rollouts that keep the bend stiff are
chaotic in float32 and are checked over one substep, longer rollouts with softer bends or none."""
import numpy as np
import pytest

torch = pytest.importorskip("torch")

from oracle import diff_ref as R
from tests.helpers import bits
from xrtailor_gb300 import ClothSolver, XrtError, scenes

pytestmark = pytest.mark.gpu


def _setup(n=16, obstacle=False, seed=0, substeps=3, iterations=4, passes=1, bending=True,
           bend_compliance=1e-5, tile=None):
    # with the obstacle the sheet starts 5 mm into the sphere's cap: VF, RT and EE records
    cloth = scenes.grid_cloth(n, 0.4, origin=(0.3, 0.295 if obstacle else 0.6, 0.3),
                              jitter=1e-3, seed=seed + 1)
    pins = scenes.two_corner_pins(n)
    cloth.fixed_indices = pins
    cloth.attached_indices = pins
    p = scenes._params(num_substeps=substeps, num_iterations=iterations,
                       stretch_compliance=1e-7, bend_compliance=bend_compliance,
                       enable_self_collision=0, solve_bending=int(bending),
                       num_collision_passes=passes, update_obstacle_animation=0)
    s = ClothSolver(p)
    if tile is not None:
        s.set_tile_vertices(tile)
    s.add_cloth(cloth, particle_diameter=0.02)
    obs = None
    if obstacle:
        obs = scenes.icosphere(2, 0.3, center=(0.5, 0.0, 0.5))
        s.add_obstacle(obs)
    s.start()
    sz = s.sizes()
    V, E, B = sz.num_vertices, sz.num_edges, sz.num_bends
    rng = np.random.default_rng(seed)
    comp = np.exp(rng.uniform(np.log(1e-8), np.log(1e-5), E)).astype(np.float32)
    bcomp = np.exp(rng.uniform(np.log(0.3 * bend_compliance), np.log(3 * bend_compliance),
                               B)).astype(np.float32)
    mass = rng.uniform(0.5, 2.0, V).astype(np.float32)
    pinned = np.zeros(V, bool)
    pinned[pins] = True
    w = np.where(pinned, 0.0, 1.0 / mass).astype(np.float32)
    v0 = rng.normal(0.0, 0.05, (V, 3)).astype(np.float32)
    s.set_compliance(0, comp)
    if B:
        s.set_compliance(1, bcomp)
    s.set_inv_mass(w)
    s.set_state(cloth.positions, v0)
    return s, p, obs, pinned, dict(comp=comp, bcomp=bcomp, mass=mass, v0=v0,
                                   x0=cloth.positions.astype(np.float32))


def _rel(a, b):
    return float(np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-30))


KEYS = ("position", "velocity", "mass", "stretch_compliance", "bend_compliance")


def _check(s, p, pinned, a, c, contacts, cv=None, factor=4.0, floor=2e-4, forward=1e-4, g=None,
           same_program=None):
    """Run the library's reverse pass (or take its gradients `g`) and compare with the
    reference in float64 (and float32 for the error floor).  `same_program`: bound on the
    relative error against the float32 autodiff of the same program (whose trajectory follows
    the library's where the frame is well conditioned).  Returns the relative errors."""
    xf = s.host_positions()
    if g is None:
        g = s.backward(c, cv)
    prob = R.problem_from(s, p, a["bcomp"])
    prob.w_pinned = pinned
    prob.contacts = contacts
    args = (a["x0"], a["v0"], a["mass"], a["comp"], prob.bend_compliance, prob, c, cv)
    g64, x64 = R.gradients(*args)
    with R.precision(torch.float32):
        g32, x32 = R.gradients(*args)
    dx, dx32 = np.abs(xf - x64).max(), np.abs(x32 - x64).max()
    assert dx < max(forward, factor * dx32), ("float32 forward left the float64 trajectory",
                                               dx, dx32)
    free = ~pinned
    errs = {}
    for k in KEYS:
        if k == "bend_compliance" and not len(prob.bend_compliance):
            continue
        sel = free if k == "mass" else slice(None)
        e = _rel(g[k][sel], g64[k][sel])
        e32 = _rel(g32[k][sel], g64[k][sel])
        errs[k] = (e, e32, _rel(g[k][sel], g32[k][sel]))
        assert e <= max(factor * e32, floor), (k, e, e32)
        if same_program is not None:
            assert errs[k][2] <= same_program, (k, errs[k])
    # the state after the reverse pass is the state before it
    np.testing.assert_array_equal(bits(s.host_positions()), bits(xf))
    return errs


# schedules: the default tiles, small tiles (many tile colors: the tiled replay and reverse
# launch per tile color), none (one launch per color)
TILES = [None, 32, 0]


@pytest.mark.parametrize("tile", TILES)
def test_adjoint_matches_fp64_reference_without_bending(xrt, tile):
    """Two frames of 3 substeps x 4 iterations: stretch, LRA, predict, finalize."""
    s, p, obs, pinned, a = _setup(n=16, bending=False, tile=tile)
    s.diff_begin()
    s.step()
    s.step()
    c = np.random.default_rng(5).normal(size=(len(a["x0"]), 3)).astype(np.float32)
    _check(s, p, pinned, a, c, [[None], [None]], same_program=1e-4)


@pytest.mark.parametrize("tile", TILES)
def test_adjoint_matches_fp64_reference_with_stiff_bending_one_substep(xrt, tile):
    s, p, obs, pinned, a = _setup(n=16, substeps=1, iterations=1, bend_compliance=1e-5,
                                  tile=tile)
    s.diff_begin()
    s.step()
    c = np.random.default_rng(6).normal(size=(len(a["x0"]), 3)).astype(np.float32)
    _check(s, p, pinned, a, c, [[None]])


@pytest.mark.parametrize("tile", TILES)
def test_adjoint_matches_fp64_reference_with_soft_bending(xrt, tile):
    s, p, obs, pinned, a = _setup(n=16, substeps=2, iterations=2, bend_compliance=1e-2,
                                  tile=tile)
    s.diff_begin()
    s.step()
    c = np.random.default_rng(7).normal(size=(len(a["x0"]), 3)).astype(np.float32)
    # four bend sweeps on a folding sheet: the float32 trajectories (library, torch) part
    # further than in the other cases, hence the wider multiple of the float32 floor
    _check(s, p, pinned, a, c, [[None]], factor=6.0)


def test_adjoint_matches_fp64_reference_with_obstacle_contacts(xrt):
    s, p, obs, pinned, a = _setup(n=16, obstacle=True, substeps=2, iterations=2, passes=1,
                                  bending=False)
    s.diff_begin()
    s.step()
    # one collision pass per frame: the contacts now held are the pass's
    ct = R.contacts_from_export(s.export_contacts(), obs.positions, obs.triangles)
    assert (ct.vf_idx >= 0).sum() + (ct.rt_idx >= 0).sum() > 0, "the scene has no contact"
    assert (ct.ee_a[:, 0] <= 1e6).sum() > 0, "the scene has no edge contact"
    c = np.random.default_rng(8).normal(size=(len(a["x0"]), 3)).astype(np.float32)
    _check(s, p, pinned, a, c, [[ct]], same_program=1e-4)


def test_torch_rollout_gradients(xrt):
    """xrtailor_gb300.diff.rollout: a loss on final positions and velocities through
    torch.autograd gives the library's reverse pass, and that matches the reference."""
    from xrtailor_gb300.diff import rollout
    s, p, obs, pinned, a = _setup(n=16, obstacle=True, substeps=2, iterations=2, passes=1,
                                  bending=False)
    ct = None
    rng = np.random.default_rng(10)
    V = len(a["x0"])
    c, cv = (rng.normal(size=(V, 3)).astype(np.float32) for _ in range(2))
    t = {k: torch.tensor(a[k], requires_grad=True) for k in ("x0", "v0", "mass", "comp")}
    x, v = rollout(s, 1, t["x0"], t["v0"], t["mass"], t["comp"])
    ct = R.contacts_from_export(s.export_contacts(), obs.positions, obs.triangles)
    ((x * torch.from_numpy(c)).sum() + (v * torch.from_numpy(cv)).sum()).backward()
    g = dict(position=t["x0"].grad.numpy(), velocity=t["v0"].grad.numpy(),
             mass=t["mass"].grad.numpy(), stretch_compliance=t["comp"].grad.numpy(),
             bend_compliance=np.zeros(0))
    np.testing.assert_array_equal(bits(x.detach().numpy()), bits(s.host_positions()))
    _check(s, p, pinned, a, c, [[ct]], cv=cv, g=g, same_program=1e-4)


def test_batched_adjoint_matches_single_contexts(xrt):
    """Three instances of different sizes in one context: each instance's gradients are those
    of a context holding that instance alone (the same replay; only the order of the atomic
    source-share and edge-contact sums differs)."""
    sizes = (10, 13, 16)
    p = scenes._params(num_substeps=2, num_iterations=3, stretch_compliance=1e-7,
                       bend_compliance=1e-3, enable_self_collision=0, num_collision_passes=2,
                       update_obstacle_animation=0)
    rng = np.random.default_rng(11)
    items = []
    for k, n in enumerate(sizes):
        cloth = scenes.grid_cloth(n, 0.4, origin=(0.3, 0.295, 0.3), jitter=1e-3, seed=20 + k)
        pins = scenes.two_corner_pins(n)
        cloth.fixed_indices = pins
        cloth.attached_indices = pins
        obs = scenes.icosphere(2, 0.3, center=(0.5, 0.0, 0.5))
        items.append((cloth, obs, pins))
    batch = ClothSolver(p)
    for cloth, obs, _ in items:
        batch.add_instance(cloth, obs, particle_diameter=0.02)
    batch.start()
    singles = []
    for cloth, obs, _ in items:
        s = ClothSolver(p)
        s.add_cloth(cloth, particle_diameter=0.02)
        s.add_obstacle(obs)
        s.start()
        singles.append(s)
    data = []
    for (cloth, obs, pins), s in zip(items, singles):
        sz = s.sizes()
        V = sz.num_vertices
        comp = np.exp(rng.uniform(np.log(1e-8), np.log(1e-5), sz.num_edges)).astype(np.float32)
        bcomp = np.exp(rng.uniform(np.log(1e-4), np.log(1e-2), sz.num_bends)).astype(np.float32)
        w = (1.0 / rng.uniform(0.5, 2.0, V)).astype(np.float32)
        w[pins] = 0.0
        v0 = rng.normal(0.0, 0.05, (V, 3)).astype(np.float32)
        c = rng.normal(size=(V, 3)).astype(np.float32)
        for solver in (s,):
            solver.set_compliance(0, comp)
            solver.set_compliance(1, bcomp)
            solver.set_inv_mass(w)
            solver.set_state(cloth.positions, v0)
        data.append((comp, bcomp, w, v0, c))
    cat = lambda j: np.concatenate([d[j] for d in data])  # noqa: E731
    batch.set_compliance(0, cat(0))
    batch.set_compliance(1, cat(1))
    batch.set_inv_mass(cat(2))
    batch.set_state(np.concatenate([it[0].positions for it in items]), cat(3))
    for solver in singles + [batch]:
        solver.diff_begin()
        solver.step()
        solver.step()
    gb = batch.backward(cat(4))
    vb = eb = bb = 0
    for s, d in zip(singles, data):
        sz = s.sizes()
        gs = s.backward(d[4])
        sl = {"position": slice(vb, vb + sz.num_vertices), "velocity": slice(vb, vb + sz.num_vertices),
              "mass": slice(vb, vb + sz.num_vertices),
              "stretch_compliance": slice(eb, eb + sz.num_edges),
              "bend_compliance": slice(bb, bb + sz.num_bends)}
        for k in KEYS:
            np.testing.assert_allclose(gb[k][sl[k]], gs[k], rtol=2e-4,
                                       atol=2e-5 * np.abs(gs[k]).max(), err_msg=k)
        vb += sz.num_vertices
        eb += sz.num_edges
        bb += sz.num_bends


@pytest.mark.parametrize("tile", TILES)
def test_backward_leaves_the_rollout_unchanged(xrt, tile):
    """Stepping on after a reverse pass gives the same bits as a context that never ran one."""
    s, p, obs, pinned, a = _setup(n=16, obstacle=True, passes=3, tile=tile)
    t, _, _, _, _ = _setup(n=16, obstacle=True, passes=3, tile=tile)
    s.diff_begin()
    for solver in (s, t):
        solver.step()
        solver.step()
    s.backward(np.ones((s.sizes().num_vertices, 3), np.float32))
    s.diff_end()
    for solver in (s, t):
        solver.step()
    np.testing.assert_array_equal(bits(s.host_positions()), bits(t.host_positions()))


def test_backward_is_deterministic(xrt):
    s, p, obs, pinned, a = _setup(n=10, obstacle=True, passes=2)
    s.diff_begin()
    s.step()
    c = np.random.default_rng(9).normal(size=(len(a["x0"]), 3)).astype(np.float32)
    g1 = s.backward(c)
    g2 = s.backward(c)
    for k in KEYS:
        assert np.isfinite(g1[k]).all(), k
        np.testing.assert_allclose(g1[k], g2[k], rtol=1e-5, atol=1e-9 * np.abs(g1[k]).max())


def test_adjoint_rejects_unsupported_frames(xrt):
    cloth = scenes.grid_cloth(8, 0.4, origin=(0.0, 0.5, 0.0))
    p = scenes._params(num_substeps=2, num_iterations=2, num_collision_passes=1,
                       enable_self_collision=1)
    s = ClothSolver(p)
    s.add_cloth(cloth, particle_diameter=0.02)
    s.start()
    with pytest.raises(XrtError):
        s.diff_begin()
    with pytest.raises(XrtError):
        s.backward(np.zeros((64, 3), np.float32))


@pytest.mark.parametrize("frames_per_checkpoint", [2, 3])
def test_checkpoint_interval_gives_the_same_gradients(xrt, frames_per_checkpoint):
    """Checkpoints every k substeps (k a multiple of the frame's substeps): the reverse pass
    recomputes the frames between checkpoints with the forward itself, so the gradients are
    those of per-frame checkpoints (up to the order of the atomic source-share sums), and the
    rollout after the reverse pass is unchanged."""
    runs = []
    for interval in (None, frames_per_checkpoint):
        s, p, obs, pinned, a = _setup(n=12, obstacle=True, substeps=2, iterations=3, passes=2)
        s.diff_begin(None if interval is None else interval * p.num_substeps)
        for _ in range(5):
            s.step()
        x_end = s.host_positions()
        c = np.random.default_rng(12).normal(size=(len(a["x0"]), 3)).astype(np.float32)
        g = s.backward(c)
        np.testing.assert_array_equal(bits(s.host_positions()), bits(x_end))
        runs.append(g)
    for k in KEYS:
        assert np.isfinite(runs[1][k]).all(), k
        np.testing.assert_allclose(runs[1][k], runs[0][k], rtol=1e-5,
                                   atol=1e-9 * np.abs(runs[0][k]).max(), err_msg=k)


def test_checkpoint_interval_must_be_a_multiple_of_the_frame(xrt):
    s, p, obs, pinned, a = _setup(n=8, substeps=3, iterations=2)
    for bad in (0, -3, 4):
        with pytest.raises(XrtError):
            s.diff_begin(bad)
    s.diff_begin(6)
    s.diff_end()


def test_adjoint_matches_fp64_central_differences_on_a_smooth_rollout(xrt):
    """A well-conditioned rollout (soft stretch, compliance 1e-4 to 1e-3, no bend, no contact):
    two frames of 3 substeps x 4 iterations with LRA.  The library's float32 gradients, projected
    on 50 random directions r (relative for mass and compliance, absolute for velocity), match
    FP64 central differences (h = 1e-6) of the reference program within 1e-4 of the directional
    derivative's scale: |fd - g.r| <= 1e-4 * ||g * s||, where s is the per-component scale of r
    (so ||g * s|| is the RMS of g.r over such directions; a single direction can be nearly
    orthogonal to g, and then |g.r| itself is no measure of the error)."""
    s, p, obs, pinned, a = _setup(n=12, bending=False)
    rng = np.random.default_rng(21)
    E = s.sizes().num_edges
    comp = np.exp(rng.uniform(np.log(1e-4), np.log(1e-3), E)).astype(np.float32)
    s.set_compliance(0, comp)
    s.set_state(a["x0"], a["v0"])
    s.diff_begin()
    s.step()
    s.step()
    c = rng.normal(size=(len(a["x0"]), 3)).astype(np.float32)
    g = s.backward(c)
    prob = R.problem_from(s, p, a["bcomp"])
    prob.w_pinned = pinned
    prob.contacts = [[None], [None]]
    x0, v0, mass = (np.asarray(a[k], np.float64) for k in ("x0", "v0", "mass"))
    comp64, bcomp64 = comp.astype(np.float64), np.asarray(prob.bend_compliance, np.float64)
    free = ~pinned

    def L(dv, dm, dc):
        with torch.no_grad():
            x = R.rollout(*(torch.as_tensor(v, dtype=torch.float64) for v in
                            (x0, v0 + dv, mass + dm, comp64 + dc, bcomp64)), prob)
        return float((x.numpy() * c).sum())

    h = 1e-6
    worst = 0.0
    for k in range(50):
        rv = rng.normal(size=v0.shape)
        rm = mass * rng.normal(size=mass.shape) * free
        rc = comp64 * rng.normal(size=comp64.shape)
        fd = (L(h * rv, h * rm, h * rc) - L(-h * rv, -h * rm, -h * rc)) / (2 * h)
        ad = float((g["velocity"].astype(np.float64) * rv).sum() +
                   (g["mass"].astype(np.float64) * rm).sum() +
                   (g["stretch_compliance"].astype(np.float64) * rc).sum())
        scale = float(np.sqrt((g["velocity"].astype(np.float64) ** 2).sum() +
                              ((g["mass"].astype(np.float64) * mass * free) ** 2).sum() +
                              ((g["stretch_compliance"].astype(np.float64) * comp64) ** 2).sum()))
        err = abs(fd - ad) / scale
        worst = max(worst, err)
        assert err <= 1e-4, (k, fd, ad, scale, err)
