"""Differentiable rollout on the GPU (cf_rollout_* / cf_rdf*) against the FP64
oracle: its analytic adjoint, FP64 central finite differences, and the soft
radial distribution and its gradient.

Tolerances: gradients within 1e-3 relative of the FP64 references (per entry
for the force table and the step parameters, with a floor of 1e-3 of the
largest entry; norm-wise and for 99.5% of particles for position
gradients, since a particle in a pair within FP32 rounding of its cutoff
can have a different neighbour set in the FP32 and FP64 trajectories), and
within 1e-4 of the FP64 adjoint evaluated along the GPU's own trajectory.
Finite differences use eps = 1e-6 and skip a sample whose two rollouts
differ in some step's neighbour counts (it straddles a cutoff)."""

import numpy as np
import pytest

import oracle
from cellflow_gb300 import inputs
from cellflow_gb300._lib import CellFlowError
from cellflow_gb300.world import ParticleSimulation

pytestmark = pytest.mark.gpu

torch = pytest.importorskip("torch")


def make_world(n, T, radius, seed, vel_sigma=0.0):
    w = inputs.Workload("adj", n=n, num_types=T, radius=radius, steps=1, seed=seed)
    params = w.params()
    pos, types, table = w.positions(), w.types(), w.table()
    vel = (np.random.default_rng(seed).normal(0.0, vel_sigma, size=(n, 3)).astype(np.float32)
           if vel_sigma else np.zeros((n, 3), np.float32))
    sim = ParticleSimulation(n, T, 2.0, 2.0, 2.0)
    sim.set_particles(pos, types, vel)
    sim.setForceTable(table)
    sim.setRadioByType(np.zeros(T, np.float32))
    return sim, params, pos, vel, types, table


def dev4(a):
    """(n, 4) device copy; synchronised, since the world runs on its own non-blocking stream."""
    t = torch.zeros((len(a), 4), dtype=torch.float32, device="cuda")
    t[:, :3] = torch.from_numpy(np.ascontiguousarray(a, np.float32)).cuda()
    torch.cuda.synchronize()
    return t


def close_entries(g, ref, rel=1e-3):
    floor = rel * np.abs(ref).max()
    return np.abs(g - ref) <= rel * np.abs(ref) + floor


def test_rollout_forward_equals_plain_steps(cflib):
    sim_a, params, pos, vel, types, table = make_world(3000, 5, 0.15, 3, 0.02)
    sim_b, *_ = make_world(3000, 5, 0.15, 3, 0.02)
    sim_a.rollout_forward(params, 9, 4)
    sim_b.simulate(params, 9)
    for x, y in zip(sim_a.get_state(), sim_b.get_state()):
        assert np.array_equal(x, y)


@pytest.mark.parametrize("every", [3, 16])
def test_rollout_gradient_matches_oracle_adjoint(cflib, every):
    n, T, K = 2048, 6, 8
    sim, params, pos, vel, types, table = make_world(n, T, 0.3, 11, 0.05)
    rng = np.random.default_rng(5)
    wx, wv = rng.normal(size=(n, 3)).astype(np.float32), rng.normal(size=(n, 3)).astype(np.float32)
    sim.rollout_forward(params, K, every)
    gx0 = torch.empty((n, 4), dtype=torch.float32, device="cuda")
    gv0 = torch.empty_like(gx0)
    gx, gv = dev4(wx), dev4(wv)
    gF, gp = sim.rollout_backward(gx.data_ptr(), gv.data_ptr(), gx0.data_ptr(), gv0.data_ptr())
    torch.cuda.synchronize()
    eff = oracle.eff_table(params, np.zeros(T, np.float32), T)
    o0, ov0, oF, op = oracle.rollout_grad_f64(pos, vel, types, np.zeros(n, np.int32), table, eff, params, K,
                                              wx, wv)
    assert close_entries(gF, oF).all(), np.abs(gF - oF).max() / np.abs(oF).max()
    assert np.all(np.abs(gp - op) <= 1e-3 * np.abs(op) + 1e-6), (gp, op)
    g0 = gx0[:, :3].cpu().numpy()
    v0 = gv0[:, :3].cpu().numpy()
    for g, o in ((g0, o0), (v0, ov0)):
        assert np.linalg.norm(g - o) <= 1e-3 * np.linalg.norm(o)
        per = np.linalg.norm(g - o, axis=1) <= 1e-3 * np.linalg.norm(o, axis=1) + 1e-3 * np.sqrt(np.mean(o * o))
        assert per.mean() >= 0.995


def test_checkpoint_interval_does_not_change_gradients(cflib):
    n, T, K = 4096, 4, 8
    out = []
    for every in (1, 3, 8):
        sim, params, *_ = make_world(n, T, 0.2, 7, 0.05)
        sim.rollout_forward(params, K, every)
        gx = dev4(np.ones((n, 3), np.float32))
        g0 = torch.empty((n, 4), dtype=torch.float32, device="cuda")
        gF, gp = sim.rollout_backward(gx.data_ptr(), None, g0.data_ptr(), None)
        torch.cuda.synchronize()
        out.append((g0[:, :3].cpu().numpy(), gF, gp))
        sim.close()
    for g0, gF, gp in out[1:]:
        np.testing.assert_allclose(g0, out[0][0], rtol=1e-5, atol=1e-6 * np.abs(out[0][0]).max())
        np.testing.assert_allclose(gF, out[0][1], rtol=1e-5, atol=1e-6 * np.abs(out[0][1]).max())
        np.testing.assert_allclose(gp, out[0][2], rtol=1e-5)


def test_rollout_graphs_follow_scratch_reallocation(cflib):
    """The rollout's forward and backward run as cached CUDA graphs that read the
    cell-list scratch by address.  Proximity calls on much finer grids grow that
    scratch between rollouts of the same shape; the rollouts after them must not
    replay a graph holding the freed buffers: their states and gradients equal
    those of a world whose scratch never moved."""
    n, T, K, every = 3000, 4, 6, 3
    sim, params, *_ = make_world(n, T, 0.15, 21, 0.03)
    ref, *_ = make_world(n, T, 0.15, 21, 0.03)
    start = sim.get_state()
    gx = dev4(np.ones((n, 3), np.float32))

    def rollout(s, between=None):
        s.set_state(*start)
        s.rollout_forward(params, K, every)
        if between is not None:
            s.proximity_edges(between, 3)  # offsets and tile totals reallocated for the finer grid
        g0 = torch.empty((n, 4), dtype=torch.float32, device="cuda")
        gF, gp = s.rollout_backward(gx.data_ptr(), None, g0.data_ptr(), None)
        torch.cuda.synchronize()
        return s.get_state(), g0[:, :3].cpu().numpy(), gF, gp

    first = rollout(sim)
    sim.proximity_edges(0.02, 3)  # a 100^3 grid against the step's 13^3
    again = rollout(sim, between=0.008)  # the 4M-cell cap, between the forward and the backward
    want = rollout(ref)
    for got in (first, again):
        for x, y in zip(got[0], want[0]):
            assert np.array_equal(x, y)
        for g, r in zip(got[1:], want[1:]):  # table gradients sum double atomics: order may differ
            np.testing.assert_allclose(g, r, rtol=1e-6, atol=1e-7 * np.abs(r).max())


def test_backward_state_is_the_forward_state(cflib):
    sim, params, *_ = make_world(2000, 3, 0.2, 9, 0.05)
    sim.rollout_forward(params, 5, 2)
    after = sim.get_state()
    gx = dev4(np.ones((2000, 3), np.float32))
    sim.rollout_backward(gx.data_ptr(), None, None, None)
    for x, y in zip(after, sim.get_state()):
        assert np.array_equal(x, y)


def test_rdf_matches_oracle(cflib):
    n, T, bins, rmax = 8192, 3, 32, 0.2
    sim, params, pos, vel, types, table = make_world(n, T, 0.1, 4)
    hist = torch.empty((T, T, bins), dtype=torch.float32, device="cuda")
    sim.rdf(bins, rmax, hist.data_ptr())
    torch.cuda.synchronize()
    ref = oracle.rdf_f64(pos, types, T, [2.0, 2.0, 2.0], bins, rmax)
    np.testing.assert_allclose(hist.cpu().numpy(), ref, rtol=2e-4, atol=2e-4 * np.abs(ref).max())
    rng = np.random.default_rng(1)
    gh = rng.normal(size=(T, T, bins)).astype(np.float32)
    ghd = torch.from_numpy(gh).cuda()
    g4 = torch.empty((n, 4), dtype=torch.float32, device="cuda")
    torch.cuda.synchronize()
    sim.rdf_backward(bins, rmax, ghd.data_ptr(), g4.data_ptr())
    torch.cuda.synchronize()
    gref = oracle.rdf_grad_f64(pos, types, T, [2.0, 2.0, 2.0], bins, rmax, gh)
    g = g4[:, :3].cpu().numpy()
    assert np.linalg.norm(g - gref) <= 1e-4 * np.linalg.norm(gref)


def rdf_loss_case(n=16384, T=6, K=8, seed=0x5EED0005):
    """The differentiable-rollout configuration: uniform positions, radius 0.1, target the
    radial distribution after K steps under a hidden seeded force table."""
    sim, params, pos, vel, types, table = make_world(n, T, 0.1, seed)
    hidden = inputs.gaussian_table(T, 0.0, 0.5, seed + 1)
    eff = oracle.eff_table(params, np.zeros(T, np.float32), T)
    xs, *_ = oracle.rollout_f64(pos, vel, types, np.zeros(n, np.int32), hidden, eff, params, K)
    target = oracle.rdf_f64(xs, types, T, [2.0, 2.0, 2.0], 32, 0.2)
    return sim, params, pos, vel, types, table, eff, target


def gpu_rdf_loss_grads(K, n=16384, T=6, every=4):
    """Gradients of the RDF loss through the torch binding, plus the FP32 trajectory the
    GPU stepped through (states before every step and after the last)."""
    from cellflow_gb300 import autograd as cfa

    sim, params, pos, vel, types, table, eff, target = rdf_loss_case(n, T, K)
    s0 = sim.get_state()
    P, V, Cn = [], [], []
    for s in range(K + 1):
        p4, v4, c = sim.get_state()
        P.append(p4[:, :3].astype(np.float64))
        V.append(v4[:, :3].astype(np.float64))
        Cn.append(c)
        if s < K:
            sim.simulate(params, 1)
    sim.set_state(*s0)
    x0 = torch.from_numpy(pos).cuda().requires_grad_(True)
    v0 = torch.zeros((n, 3), dtype=torch.float32, device="cuda", requires_grad=True)
    F = torch.from_numpy(table.copy()).requires_grad_(True)
    phys = cfa.phys_tensor(params).requires_grad_(True)
    xk, _ = cfa.rollout(x0, v0, F, phys, sim, params, K, every)
    assert np.array_equal(xk.detach().cpu().numpy(), P[-1].astype(np.float32))
    h = cfa.radial_distribution(xk, sim, 32, 0.2)
    loss = ((h - torch.from_numpy(target).float().cuda()) ** 2).mean()
    loss.backward()
    case = dict(params=params, pos=pos, vel=vel, types=types, table=table, eff=eff, target=target, n=n, T=T, K=K)
    grads = dict(F=F.grad.numpy().astype(np.float64), phys=phys.grad.numpy(), x0=x0.grad.cpu().numpy())
    return case, grads, (np.stack(P), np.stack(V), np.stack(Cn))


def oracle_rdf_loss_grads(case, traj=None):
    """FP64 adjoint of the RDF loss, along the given trajectory or the oracle's own."""
    c = case
    ext = [2.0, 2.0, 2.0]
    if traj is None:
        xK, *_ = oracle.rollout_f64(c["pos"], c["vel"], c["types"], np.zeros(c["n"], np.int32), c["table"], c["eff"],
                                    c["params"], c["K"])
    else:
        xK = traj[0][-1]
    h = oracle.rdf_f64(xK, c["types"], c["T"], ext, 32, 0.2)
    gxK = oracle.rdf_grad_f64(xK, c["types"], c["T"], ext, 32, 0.2, 2.0 * (h - c["target"]) / h.size)
    zero = np.zeros((c["n"], 3))
    if traj is None:
        g0, _, gF, gp = oracle.rollout_grad_f64(c["pos"], c["vel"], c["types"], np.zeros(c["n"], np.int32),
                                                c["table"], c["eff"], c["params"], c["K"], gxK, zero)
    else:
        g0, _, gF, gp = oracle.rollout_grad_traj_f64(*traj, c["types"], c["table"], c["eff"], c["params"], gxK, zero)
    return dict(F=gF, phys=gp, x0=g0)


def finite_differences(case, which, eps=1e-6):
    """FP64 central differences of the RDF loss; None where the two rollouts' neighbour
    counts differ at some step (the difference straddles a cutoff)."""
    c = case

    def L(F_=c["table"], x_=c["pos"], **override):
        x, _, _, _, fp = oracle.rollout_f64(x_, c["vel"], c["types"], np.zeros(c["n"], np.int32), F_, c["eff"],
                                            c["params"], c["K"], **override)
        h = oracle.rdf_f64(x, c["types"], c["T"], [2.0, 2.0, 2.0], 32, 0.2)
        return float(np.mean((h - c["target"]) ** 2)), fp

    out = {}
    for key in which:
        kind, idx = key
        if kind == "F":
            Fp, Fm = c["table"].astype(np.float64), c["table"].astype(np.float64)
            Fp[idx] += eps
            Fm[idx] -= eps
            (lp, a), (lm, b) = L(F_=Fp), L(F_=Fm)
        elif kind == "phys":
            name = oracle.GRAD_PARAMS[idx]
            v = getattr(c["params"], name)
            (lp, a), (lm, b) = L(**{name: v + eps}), L(**{name: v - eps})
        else:
            xp, xm = c["pos"].astype(np.float64), c["pos"].astype(np.float64)
            xp[idx] += eps
            xm[idx] -= eps
            (lp, a), (lm, b) = L(x_=xp), L(x_=xm)
        out[key] = (lp - lm) / (2 * eps) if a == b else None
    return out


def fd_keys(case, n_pos=8):
    T = case["T"]
    rng = np.random.default_rng(3)
    keys = [("F", (a, b)) for a in range(T) for b in range(T)]
    keys += [("phys", k) for k in range(len(oracle.GRAD_PARAMS))]
    keys += [("x0", (int(i), int(rng.integers(3)))) for i in rng.choice(case["n"], n_pos, replace=False)]
    return keys


def assert_matches(grads, ref, rel, keys=None, what=""):
    """Per entry: |g - r| <= rel |r| + rel * (largest |r| of its group)."""
    for group in ("F", "phys", "x0"):
        g, r = np.asarray(grads[group], np.float64), np.asarray(ref[group], np.float64)
        floor = rel * np.abs(r).max() if group != "phys" else 1e-12
        bad = np.abs(g - r) > rel * np.abs(r) + floor
        assert not bad.any(), f"{what} {group}: worst {np.abs(g - r)[bad].max()} of scale {np.abs(r).max()}"


def test_rdf_loss_gradient_equals_fp64_adjoint_on_the_same_trajectory(cflib):
    """The C5 configuration at K = 8: the GPU adjoint (FP32 kernels, through the torch
    binding) against the FP64 adjoint along the very states the GPU stepped through."""
    case, grads, traj = gpu_rdf_loss_grads(8)
    ref = oracle_rdf_loss_grads(case, traj)
    assert_matches(grads, ref, 1e-4, what="GPU vs FP64 adjoint on the GPU trajectory")


def test_rdf_loss_gradient_matches_finite_differences_short_rollout(cflib):
    """K = 2, where the FP32 and FP64 trajectories still agree to ~1e-6: the GPU gradient
    against FP64 central finite differences (eps = 1e-6) within 1e-3."""
    case, grads, _ = gpu_rdf_loss_grads(2)
    fd = finite_differences(case, fd_keys(case))
    excluded = sum(v is None for v in fd.values())
    assert excluded <= 3
    for group in ("F", "phys", "x0"):
        items = [(k, v) for k, v in fd.items() if k[0] == group and v is not None]
        scale = max(abs(v) for _, v in items)
        for (kind, idx), v in items:
            g = grads[kind][idx]
            tol = 1e-3 * abs(v) + (1e-3 * scale if group != "phys" else 0.0)
            assert abs(g - v) <= tol, (kind, idx, g, v)


# Measured relative gaps between the GPU's step-parameter gradients at K = 8 and FP64
# finite differences (the FP32 and FP64 trajectories diverge, see the test below), with
# headroom; a gap above its bound is a change in the adjoint, not rounding.
# Measured on a GB300: repulsion 1.78e-2, attraction 6.6e-4, k 6.2e-3, force multiplier 1.9e-3,
# balance 3.4e-3, friction 3.8e-4; the bounds are twice those.
K8_PARAM_GAP = {"repulsion": 0.036, "attraction": 0.0014, "k": 0.0125, "force_multiplier": 0.004, "balance": 0.007,
                "friction": 0.0008}


def test_rdf_loss_gradient_k8_decomposition(cflib):
    """K = 8.  The reference's parameters make close pairs stiff for explicit Euler at
    dt = 0.01, so the FP32 and FP64 rollouts drift apart (1e-4 in position by step 8) and
    their gradients differ by more than 1e-3 for some step parameters.  The check splits
    the comparison: FP64 adjoint = FP64 finite differences (1e-4), GPU = FP64 adjoint on
    the GPU's own trajectory (1e-4, above), and the force-table and position gradients of
    the two trajectories agree within 1e-3."""
    case, grads, traj = gpu_rdf_loss_grads(8)
    own = oracle_rdf_loss_grads(case)
    keys = fd_keys(case)
    fd = finite_differences(case, keys)
    assert sum(v is None for v in fd.values()) <= 3
    for (kind, idx), v in fd.items():
        if v is None:
            continue
        r = own[kind][idx]
        scale = np.abs(own[kind]).max() if kind != "phys" else 0.0
        assert abs(r - v) <= 1e-4 * abs(v) + 1e-5 * scale, (kind, idx, r, v)
    g, r = grads["F"], own["F"]
    assert np.all(np.abs(g - r) <= 1e-3 * np.abs(r) + 1e-3 * np.abs(r).max())
    assert np.linalg.norm(grads["x0"] - own["x0"]) <= 2e-3 * np.linalg.norm(own["x0"])
    # the six step parameters: the GPU gradient against FP64 finite differences of the FP64
    # rollout differs by the FP32/FP64 trajectory divergence, tracked per parameter so that a
    # change in the adjoint shows up as a change in these numbers
    gaps = {}
    for k, name in enumerate(oracle.GRAD_PARAMS):
        v = fd.get(("phys", k))
        if v is not None and v != 0.0:
            gaps[name] = abs(float(grads["phys"][k]) - v) / abs(v)
    print("\nK=8 step-parameter gradients, GPU vs FP64 finite differences (relative):",
          {k: f"{v:.2e}" for k, v in gaps.items()})
    for name, gap in gaps.items():
        assert gap <= K8_PARAM_GAP[name], (name, gap)


def test_rollout_errors(cflib):
    sim, params, *_ = make_world(500, 3, 0.2, 1)
    with pytest.raises(CellFlowError):
        sim.rollout_backward(None, None, None, None)  # no forward yet
    sim.rollout_forward(params, 3, 2)
    sim.setForceTable(np.ones((3, 3), np.float32))
    with pytest.raises(CellFlowError):
        sim.rollout_backward(None, None, None, None)  # the table changed
    with pytest.raises(CellFlowError):
        sim.rollout_forward(params, 0, 2)
    with pytest.raises(CellFlowError):
        sim.rdf(0, 0.2, 0)
