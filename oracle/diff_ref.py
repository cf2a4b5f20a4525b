"""FP64 reference of the differentiable Swift frame -- test infrastructure, not product code.

The same frame the library's hand-written adjoint differentiates (include/xrt_diff.h), restated
with torch float64 tensor operations so that torch.autograd gives reference gradients, and
checked itself against central finite differences.  Small meshes only (per-color Python loops).

Per substep (ClothSolverBase::SimulateSwift, ClothSolverBase.cpp:171-261, frames without
particle self-collision or bindings):
  predict (ClothSolverHelper.cu:125-137)
  per iteration: stretch colors in order (XPBD, lambda reset at iteration 0,
    BasicSolverHelper.cu:80-132; the library's fused multiply-adds, see _fma), bend colors in
    order (BasicSolverHelper.cu:8-72, arccos by the
    same Abramowitz & Stegun 4.4.46 polynomial as the library), LRA with pinned slots
    (LongRangeAttachments.cu:5-26), VF-CCD then VF-DCD per vertex (PBDCollision.cu:279-298, 57-80),
    EE-DCD + ApplyDeltas as a Jacobi step (PBDCollision.cu:163-212, ClothSolverHelper.cu:139-148)
  finalize (ClothSolverHelper.cu:222-236)
Contacts are inputs, held fixed per collision pass as recorded by the forward pass.
"""
import contextlib
from dataclasses import dataclass, field
from typing import List, Optional

import numpy as np
import torch

T = torch.float64


@contextlib.contextmanager
def precision(dtype):
    """Evaluate the same program in another torch dtype (float32: the error floor any
    single-precision implementation of these formulas has against the float64 one)."""
    global T
    old, T = T, dtype
    try:
        yield
    finally:
        T = old
EPS = 1e-6
ACOS_C = [-0.0012624911, 0.0066700901, -0.0170881256, 0.0308918810, -0.0501743046,
          0.0889789874, -0.2145988016, 1.5707963050]


def _sqrt0(a):
    """sqrt with a zero (not infinite) derivative at 0, so masked branches stay finite."""
    pos = a > 0
    return torch.where(pos, torch.sqrt(torch.where(pos, a, torch.ones_like(a))),
                       torch.zeros_like(a))


def acos_as(x):
    p = torch.full_like(x, ACOS_C[0])
    for c in ACOS_C[1:]:
        p = _fma(p, x, torch.full_like(x, c))
    return _sqrt0(1.0 - x) * p


def _normalize(v):
    return v / torch.sqrt((v * v).sum(-1, keepdim=True))


def _dot(a, b):
    return (a * b).sum(-1)


def _fma(a, b, c):
    """a*b + c rounded once, as the library's stretch and bend projections evaluate it (fmaf):
    in float32 through float64 and one rounding (the fused result up to a rare double rounding),
    in float64 the plain expression."""
    if T == torch.float32:
        return (a.double() * b.double() + c.double()).to(T)
    return a * b + c


def _fdot(a, b):
    """The library's fused dot product fma(a.z, b.z, fma(a.y, b.y, a.x b.x))."""
    return _fma(a[..., 2], b[..., 2], _fma(a[..., 1], b[..., 1], a[..., 0] * b[..., 0]))


@dataclass
class Contacts:
    """One collision pass: per vertex RT / VF records, per edge EE records, obstacle triangles."""
    rt_idx: np.ndarray   # V, -1 = none
    rt_qc: np.ndarray    # V x 3
    vf_idx: np.ndarray   # V
    vf_qs: np.ndarray    # V x 3
    ee_a: np.ndarray     # E x 4 {dist, p2}
    ee_b: np.ndarray     # E x 4 {q2, s}
    ee_c: np.ndarray     # E x 4 {fn, t}
    pred: np.ndarray     # F x 3 x 3 obstacle primitive vertices


@dataclass
class Problem:
    edges: np.ndarray            # E x 2 (library edge order)
    rest: np.ndarray             # E
    bends: np.ndarray            # B x 4
    theta: np.ndarray            # B
    bend_compliance: np.ndarray  # B
    s_colors: List[np.ndarray]   # stretch constraint ids per color, in execution order
    b_colors: List[np.ndarray]
    w_pinned: np.ndarray         # V bool: inverse mass 0
    lra_src: np.ndarray          # L (list order: slot-major)
    lra_tgt: np.ndarray
    lra_rest: np.ndarray
    dt: float
    substeps: int
    iterations: int
    passes: int                  # collision passes per frame
    gravity: tuple
    damping: float
    relaxation: float
    lra_stretch: float
    contacts: List[List[Optional[Contacts]]] = field(default_factory=list)  # [frame][pass]


def _stretch(x, w, lam, p: Problem, comp, reset):
    for cid in p.s_colors:
        idx = torch.as_tensor(cid)
        a = torch.as_tensor(p.edges[cid, 0])
        b = torch.as_tensor(p.edges[cid, 1])
        xa, xb = x[a], x[b]
        wa, wb = w[a], w[b]
        rest = torch.as_tensor(p.rest[cid], dtype=T)
        lam_c = torch.zeros(len(cid), dtype=T) if reset else lam[idx]
        d = xa - xb
        dist = _sqrt0(_fdot(d, d))
        mask = (dist != rest) & (wa + wb > 0)
        n = d * (1.0 / (dist + EPS))[:, None]
        at = comp[idx] / (p.dt * p.dt)
        C = dist - rest
        dl = _fma(-at, lam_c, -C) / (wa + wb + at)
        dl = torch.where(mask, dl, torch.zeros_like(dl))
        corr = dl[:, None] * n
        x = (x.index_copy(0, a, _fma(corr, wa[:, None], xa))
              .index_copy(0, b, _fma(-corr, wb[:, None], xb)))
        lam = lam.index_copy(0, idx, torch.where(mask, lam_c + dl, lam_c))
    return x, lam


def _bend(x, w, p: Problem, bcomp):
    for cid in p.b_colors:
        bi = p.bends[cid]
        i1, i2, i3, i4 = (torch.as_tensor(bi[:, k]) for k in range(4))
        x1, x2, x3, x4 = x[i1], x[i2], x[i3], x[i4]
        w1, w2, w3, w4 = w[i1], w[i2], w[i3], w[i4]
        p2, p3, p4 = x2 - x1, x3 - x1, x4 - x1
        c23, c24 = torch.cross(p2, p3, dim=-1), torch.cross(p2, p4, dim=-1)
        n1, n2 = _normalize(c23), _normalize(c24)
        d = torch.clamp(_dot(n1, n2), 0.0, 1.0)
        angle = acos_as(d)
        e23 = _sqrt0(_dot(c23, c23)) + EPS
        e24 = _sqrt0(_dot(c24, c24)) + EPS
        dd = d[:, None]
        q3 = (torch.cross(p2, n2, dim=-1) + torch.cross(n1, p2, dim=-1) * dd) / e23[:, None]
        q4 = (torch.cross(p2, n1, dim=-1) + torch.cross(n2, p2, dim=-1) * dd) / e24[:, None]
        q2 = (-(torch.cross(p3, n2, dim=-1) + torch.cross(n1, p3, dim=-1) * dd) / e23[:, None]
              - (torch.cross(p4, n1, dim=-1) + torch.cross(n2, p4, dim=-1) * dd) / e24[:, None])
        q1 = -q2 - q3 - q4
        at = bcomp[torch.as_tensor(cid)] / p.dt / p.dt
        denom = at + (w1 * _dot(q1, q1) + w2 * _dot(q2, q2) + w3 * _dot(q3, q3) +
                      w4 * _dot(q4, q4))
        ok = (angle >= EPS) & ~torch.isnan(d) & (denom >= EPS)
        s = _sqrt0(1.0 - d * d)
        theta = torch.as_tensor(p.theta[cid], dtype=T)
        lam = torch.where(ok, s * (angle - theta) / torch.where(ok, denom, torch.ones_like(denom)),
                          torch.zeros_like(denom))[:, None]
        x = (x.index_copy(0, i1, x1 + w1[:, None] * lam * q1)
              .index_copy(0, i2, x2 + w2[:, None] * lam * q2)
              .index_copy(0, i3, x3 + w3[:, None] * lam * q3)
              .index_copy(0, i4, x4 + w4[:, None] * lam * q4))
    return x


def _stage(x_in, w, p: Problem, ct: Optional[Contacts]):
    """LRA (slots in list order; sources pinned) then VF-CCD / VF-DCD; reads x_in only."""
    q = x_in
    if len(p.lra_tgt):
        slots = {}
        for k in range(len(p.lra_tgt)):
            slots.setdefault(int(p.lra_tgt[k]), []).append(k)
        depth = max(len(v) for v in slots.values())
        for r in range(depth):
            ks = np.array([v[r] for v in slots.values() if len(v) > r])
            tgt = torch.as_tensor(p.lra_tgt[ks])
            src = torch.as_tensor(p.lra_src[ks])
            xt, xs = q[tgt], x_in[src]
            target = torch.as_tensor(p.lra_rest[ks] * p.lra_stretch, dtype=T)
            skip = (w[tgt] < EPS) & (target > 0)
            diff = xt - xs
            dist = _sqrt0(_dot(diff, diff))
            on = (dist > target) & ~skip
            safe = torch.where(on, dist, torch.ones_like(dist))
            nxt = xt + (-diff + diff / safe[:, None] * target[:, None])
            q = q.index_copy(0, tgt, torch.where(on[:, None], nxt, xt))
    if ct is not None:
        pred = torch.as_tensor(ct.pred, dtype=T)
        fn = _normalize(torch.cross(pred[:, 1] - pred[:, 0], pred[:, 2] - pred[:, 0], dim=-1))
        for idx, pts, margin in ((ct.rt_idx, ct.rt_qc, 0.0), (ct.vf_idx, ct.vf_qs, 1e-3)):
            v = np.nonzero(idx >= 0)[0]
            if len(v) == 0:
                continue
            vt = torch.as_tensor(v)
            nrm = fn[torch.as_tensor(idx[v])]
            qv = q[vt]
            lam = _dot(nrm, qv - torch.as_tensor(pts[v], dtype=T)) - margin
            q = q.index_copy(0, vt, torch.where((lam < 0)[:, None], qv - lam[:, None] * nrm, qv))
    return q


def _ee(x_in, p: Problem, ct: Contacts):
    E = len(p.edges)
    a = torch.as_tensor(p.edges[:, 0])
    b = torch.as_tensor(p.edges[:, 1])
    ca = torch.as_tensor(ct.ee_a, dtype=T)
    cb = torch.as_tensor(ct.ee_b, dtype=T)
    cc = torch.as_tensor(ct.ee_c, dtype=T)
    s, t, fn = cb[:, 3], cc[:, 3], cc[:, :3]
    c1 = (1 - s)[:, None] * x_in[a] + s[:, None] * x_in[b]
    c2 = (1 - t)[:, None] * ca[:, 1:4] + t[:, None] * cb[:, :3]
    d = c1 - c2
    lam = _dot(d, fn) - 1e-3
    on = (ca[:, 0] <= 1e6) & (_sqrt0(_dot(d, d)) >= EPS) & (lam <= 0)
    lam = torch.where(on, lam, torch.zeros_like(lam))
    V = x_in.shape[0]
    delta = torch.zeros((V, 3), dtype=T)
    delta = delta.index_add(0, a, -((1 - s) * lam)[:, None] * fn)
    delta = delta.index_add(0, b, -(s * lam)[:, None] * fn)
    cnt = torch.zeros(V, dtype=T).index_add(0, a, on.to(T)).index_add(0, b, on.to(T))
    scale = torch.where(cnt > 0, p.relaxation / torch.where(cnt > 0, cnt, torch.ones_like(cnt)),
                        torch.zeros_like(cnt))
    return x_in + delta * scale[:, None]


def frame(x0, v, w, comp, bcomp, p: Problem, frame_contacts: List[Optional[Contacts]]):
    g = torch.as_tensor(p.gravity, dtype=T)
    free = (w > EPS).to(T)[:, None]
    E = len(p.edges)
    lam = torch.zeros(E, dtype=T)
    frequency = (p.substeps * p.iterations) // p.passes
    cnt = -1
    for s in range(p.substeps):
        vp = v + g * p.dt * free
        x = x0 + vp * p.dt
        for it in range(p.iterations):
            cur = s * p.iterations + it
            if cur % frequency == 0:
                cnt += 1
            ct = frame_contacts[cnt] if frame_contacts else None
            x, lam = _stretch(x, w, lam, p, comp, reset=(it == 0))
            x = _bend(x, w, p, bcomp)
            if len(p.lra_tgt) or ct is not None:
                x = _stage(x, w, p, ct)
            if ct is not None:
                x = _ee(x, p, ct)
        v = (x - x0) / p.dt * (1 - p.damping * p.dt)
        x0 = x
    return x0, v


def rollout(x0, v0, mass, comp, bcomp, p: Problem, velocity=False):
    """Final positions (and velocities) after len(p.contacts) frames (or one frame without
    contacts)."""
    w = torch.where(torch.as_tensor(p.w_pinned), torch.zeros_like(mass), 1.0 / mass)
    x, v = x0, v0
    frames = max(len(p.contacts), 1)
    for f in range(frames):
        x, v = frame(x, v, w, comp, bcomp, p, p.contacts[f] if p.contacts else [])
    return (x, v) if velocity else x


def gradients(x0, v0, mass, comp, bcomp, p: Problem, dL_dx, dL_dv=None):
    """Reference gradients of L = <dL_dx, x_final> (+ <dL_dv, v_final>) by torch.autograd
    (float64 unless run under `precision`); returned as float64 arrays."""
    args = [torch.as_tensor(np.asarray(a, np.float64), dtype=T).clone().requires_grad_(True)
            for a in (x0, v0, mass, comp, bcomp)]
    xf, vf = rollout(*args, p, velocity=True)
    L = (xf * torch.as_tensor(np.asarray(dL_dx, np.float64), dtype=T)).sum()
    if dL_dv is not None:
        L = L + (vf * torch.as_tensor(np.asarray(dL_dv, np.float64), dtype=T)).sum()
    L.backward()
    names = ("position", "velocity", "mass", "stretch_compliance", "bend_compliance")
    return {n: (a.grad.double().numpy() if a.grad is not None else np.zeros(a.shape))
            for n, a in zip(names, args)}, xf.detach().double().numpy()


def problem_from(solver, params, bend_compliance, colors=None, frames=1) -> Problem:
    """A Problem with the topology, LRA lists and (by default) the coloring a started solver
    (the library's ClothSolver or the oracle's OracleSolver) reports."""
    edges, rest = solver.edges()
    bends, theta = solver.bends()
    src, tgt, lrest = solver.lra()
    if colors is None:
        colors = (solver.coloring(0), solver.coloring(1))
    groups = [[np.nonzero(col == k)[0] for k in np.unique(col)] for col in colors]
    return Problem(
        edges=edges.astype(np.int64), rest=rest.astype(np.float64),
        bends=bends.astype(np.int64), theta=theta.astype(np.float64),
        bend_compliance=np.broadcast_to(np.asarray(bend_compliance, np.float64),
                                        (len(bends),)).copy(),
        s_colors=groups[0], b_colors=groups[1],
        w_pinned=np.zeros(0, bool),
        lra_src=src.astype(np.int64), lra_tgt=tgt.astype(np.int64),
        lra_rest=lrest.astype(np.float64),
        dt=params.frame_time / params.num_substeps, substeps=params.num_substeps,
        iterations=params.num_iterations, passes=params.num_collision_passes,
        gravity=tuple(float(g) for g in params.gravity), damping=params.damping,
        relaxation=params.relaxation_factor, lra_stretch=params.long_range_stretchiness)


def contacts_from_export(ex: dict, obstacle_positions, obstacle_triangles) -> Contacts:
    """Contacts of one collision pass from ClothSolver.export_contacts() and the obstacle."""
    ee = ex["ee"]
    op = np.asarray(obstacle_positions, np.float64)
    tri = np.asarray(obstacle_triangles, np.int64)
    return Contacts(
        rt_idx=ex["rt_index"].astype(np.int64), rt_qc=ex["rt_qc"].astype(np.float64),
        vf_idx=ex["vf_index"].astype(np.int64), vf_qs=ex["vf_qs"].astype(np.float64),
        ee_a=ee[:, 0:4].astype(np.float64),
        ee_b=np.concatenate([ee[:, 4:7], ee[:, 7:8]], 1).astype(np.float64),
        ee_c=np.concatenate([ee[:, 9:12], ee[:, 8:9]], 1).astype(np.float64),
        pred=op[tri])


def greedy_colors(idx: np.ndarray) -> List[np.ndarray]:
    """Greedy coloring in constraint order (small problems without a library export)."""
    used = {}
    col = np.zeros(len(idx), np.int64)
    for c, vs in enumerate(idx):
        taken = set()
        for v in vs:
            taken |= used.get(int(v), set())
        k = 0
        while k in taken:
            k += 1
        col[c] = k
        for v in vs:
            used.setdefault(int(v), set()).add(k)
    return [np.nonzero(col == k)[0] for k in range(col.max() + 1)]
