"""The FP64 oracle's rollout adjoint and soft radial distribution gradient against
FP64 central finite differences (no GPU).

The loss is the one the rollout is trained with, the mean squared difference
of the soft radial distribution after K steps to a target, plus a velocity
term so that the velocity adjoint is exercised.  A finite difference whose
two rollouts differ in any step's neighbour counts straddles a cutoff and is
not a derivative; such samples are excluded (and must be rare)."""

import numpy as np
import pytest

import oracle
from cellflow_gb300 import inputs

T, K, BINS, RMAX, EPS = 4, 4, 32, 0.2, 1e-6


@pytest.fixture(scope="module")
def case():
    n, seed = 600, 21
    w = inputs.Workload("adj", n=n, num_types=T, radius=0.3, steps=1, seed=seed)
    p = w.params()
    pos = w.positions().astype(np.float64)
    types = w.types()
    F = w.table().astype(np.float64)
    eff = oracle.eff_table(p, np.zeros(T, np.float32), T)
    rng = np.random.default_rng(seed)
    target = np.abs(rng.normal(1.0, 0.3, size=(T, T, BINS)))
    vel0 = rng.normal(0.0, 0.05, size=(n, 3))
    vw = rng.normal(size=(n, 3))
    return dict(n=n, p=p, pos=pos, vel=vel0, types=types, F=F, eff=eff, target=target, vw=vw)


def loss(c, pos, vel, F, **override):
    cnt = np.zeros(c["n"], np.int32)
    x, v, _, margin, fp = oracle.rollout_f64(pos, vel, c["types"], cnt, F, c["eff"], c["p"], K, **override)
    h = oracle.rdf_f64(x, c["types"], T, [2.0, 2.0, 2.0], BINS, RMAX)
    return float(np.mean((h - c["target"]) ** 2) + 0.5 * np.sum(v * c["vw"])), fp, x, v


def adjoint(c):
    L, _, x, v = loss(c, c["pos"], c["vel"], c["F"])
    h = oracle.rdf_f64(x, c["types"], T, [2.0, 2.0, 2.0], BINS, RMAX)
    gh = 2.0 * (h - c["target"]) / h.size
    gx = oracle.rdf_grad_f64(x, c["types"], T, [2.0, 2.0, 2.0], BINS, RMAX, gh)
    return oracle.rollout_grad_f64(c["pos"], c["vel"], c["types"], np.zeros(c["n"], np.int32), c["F"], c["eff"],
                                   c["p"], K, gx, 0.5 * c["vw"])


def central(c, perturb):
    lp, fpp = perturb(+EPS)
    lm, fpm = perturb(-EPS)
    return (lp - lm) / (2 * EPS), fpp == fpm


def check(fd, g, scale, what):
    assert abs(g - fd) <= 1e-4 * abs(fd) + 1e-7 * scale, f"{what}: adjoint {g!r} vs finite difference {fd!r}"


def test_oracle_adjoint_matches_finite_differences(case):
    c = case
    g0, gv0, gF, gph = adjoint(c)
    excluded = 0
    scale = np.abs(gF).max()
    for a, b in [(0, 0), (0, 3), (1, 2), (3, 1), (2, 2)]:
        def pert(e, a=a, b=b):
            F = c["F"].copy()
            F[a, b] += e
            L, fp, _, _ = loss(c, c["pos"], c["vel"], F)
            return L, fp
        fd, ok = central(c, pert)
        if not ok:
            excluded += 1
            continue
        check(fd, gF[a, b], scale, f"dL/dF[{a},{b}]")
    for k, name in enumerate(oracle.GRAD_PARAMS):
        def pert(e, name=name):
            L, fp, _, _ = loss(c, c["pos"], c["vel"], c["F"], **{name: getattr(c["p"], name) + e})
            return L, fp
        fd, ok = central(c, pert)
        if not ok:
            excluded += 1
            continue
        check(fd, gph[k], abs(fd), f"dL/d{name}")
    scale_x = np.abs(g0).max()
    for i, a in [(0, 0), (17, 2), (301, 1), (599, 0)]:
        def pert(e, i=i, a=a):
            x = c["pos"].copy()
            x[i, a] += e
            L, fp, _, _ = loss(c, x, c["vel"], c["F"])
            return L, fp
        fd, ok = central(c, pert)
        if not ok:
            excluded += 1
            continue
        check(fd, g0[i, a], scale_x, f"dL/dx0[{i},{a}]")

        def pertv(e, i=i, a=a):
            v = c["vel"].copy()
            v[i, a] += e
            L, fp, _, _ = loss(c, c["pos"], v, c["F"])
            return L, fp
        fd, ok = central(c, pertv)
        if ok:
            check(fd, gv0[i, a], np.abs(gv0).max(), f"dL/dv0[{i},{a}]")
    assert excluded <= 2


def test_rdf_gradient_matches_finite_differences(case):
    c = case
    x = c["pos"]
    h = oracle.rdf_f64(x, c["types"], T, [2.0, 2.0, 2.0], BINS, RMAX)
    gh = 2.0 * (h - c["target"]) / h.size
    g = oracle.rdf_grad_f64(x, c["types"], T, [2.0, 2.0, 2.0], BINS, RMAX, gh)

    def L(xx):
        return float(np.mean((oracle.rdf_f64(xx, c["types"], T, [2.0, 2.0, 2.0], BINS, RMAX) - c["target"]) ** 2))
    for i, a in [(3, 0), (44, 1), (500, 2)]:
        xp, xm = x.copy(), x.copy()
        xp[i, a] += EPS
        xm[i, a] -= EPS
        fd = (L(xp) - L(xm)) / (2 * EPS)
        check(fd, g[i, a], np.abs(g).max(), f"dRDF/dx[{i},{a}]")


def test_rdf_normalisation_of_uniform_gas():
    """An ideal gas has g(r) close to 1 away from r = 0 (the spline smooths the first bins)."""
    n = 20000
    pos = inputs.uniform_positions(n, 5).astype(np.float64)
    types = inputs.uniform_types(n, 2, 5)
    h = oracle.rdf_f64(pos, types, 2, [2.0, 2.0, 2.0], 16, 0.2)
    assert np.all(np.abs(h[:, :, 4:].mean(axis=2) - 1.0) < 0.05)


def test_rollout_fingerprint_detects_count_changes(case):
    c = case
    _, fp1, _, _ = loss(c, c["pos"], c["vel"], c["F"])
    _, fp2, _, _ = loss(c, c["pos"], c["vel"], c["F"])
    assert fp1 == fp2
    _, fp3, _, _ = loss(c, c["pos"], c["vel"], c["F"] * 3.0)
    assert fp3 != fp1


def test_adjoint_along_given_trajectory_equals_own(case):
    """cfo_rollout_grad_traj_f64 on the oracle's own FP64 states gives the same gradient."""
    c = case
    n = c["n"]
    P, V, Cn = [c["pos"]], [c["vel"]], [np.zeros(n, np.int32)]
    for _ in range(K):
        x, v, cnt, _, _ = oracle.rollout_f64(P[-1], V[-1], c["types"], Cn[-1], c["F"], c["eff"], c["p"], 1)
        P.append(x)
        V.append(v)
        Cn.append(cnt)
    rng = np.random.default_rng(2)
    gx, gv = rng.normal(size=(n, 3)), rng.normal(size=(n, 3))
    a = oracle.rollout_grad_f64(c["pos"], c["vel"], c["types"], np.zeros(n, np.int32), c["F"], c["eff"], c["p"], K,
                                gx, gv)
    b = oracle.rollout_grad_traj_f64(np.stack(P), np.stack(V), np.stack(Cn), c["types"], c["F"], c["eff"], c["p"],
                                     gx, gv)
    for x, y in zip(a, b):
        np.testing.assert_allclose(x, y, rtol=1e-12, atol=1e-12 * np.abs(x).max())
