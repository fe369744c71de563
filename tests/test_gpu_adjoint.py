"""Adjoint of the pair integrals (gradient with respect to vertex coordinates) through the C-ABI
and torch.autograd, against central finite differences of the CUDA forward pass and of the
oracle's forward pass (the reference's formulas on the CPU).  Loss L = sum_p c_p (P_p + w . J_p)
with seeded c_p ~ N(0, 1), w ~ N(0, 1)^3 on a radially displaced sphere (spherical harmonics of
degree <= 6, coefficients ~ N(0, 0.05^2)).  Fixed refinement and the plain Duffy potential rule
keep the forward pass a smooth function of the coordinates, so the finite differences (h = 1e-6)
have no decision jumps.  Bar: |adjoint - FD| <= 1e-6 x max |gradient| per coordinate."""
import numpy as np
import pytest

from tests._util import ensure_built

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def setup():
    torch = pytest.importorskip("torch")
    ensure_built()
    from integrator2_gb300 import meshes, pairs as P
    V, C = meshes.sh_displaced_icosphere(2, 6, 0.05, 4)
    pl = P.build_pairs(V, C)
    lists = [pl.vertex, pl.edge, pl.far, pl.self_]
    rng = np.random.default_rng(7)
    c = [rng.standard_normal(len(l)) for l in lists]
    w = rng.standard_normal(3)
    coords = rng.choice(V.size, 24, replace=False)
    return torch, V, C, lists, c, w, coords


SETTINGS = dict(mode="fixed", level=1, hard_tol=0.0)


def loss_of(torch, outs, c, w):
    L = 0.0
    for (J, P), ck in zip(outs, c):
        ck = torch.as_tensor(ck, dtype=torch.float64, device=J.device)
        L = L + (ck * (P + J @ torch.as_tensor(w, dtype=torch.float64, device=J.device))).sum()
    return L


def test_adjoint_matches_finite_differences(setup):
    torch, V, C, lists, c, w, coords = setup
    from integrator2_gb300.autograd import pair_integrals
    Vt = torch.tensor(V, dtype=torch.float64, device="cuda", requires_grad=True)
    L = loss_of(torch, pair_integrals(Vt, C, lists, **SETTINGS), c, w)
    L.backward()
    g = Vt.grad.detach().cpu().numpy().reshape(-1)
    h = 1e-6
    fd = []
    for k in coords:
        vals = []
        for s in (1.0, -1.0):
            Vp = V.copy().reshape(-1)
            Vp[k] += s * h
            Vq = torch.tensor(Vp.reshape(-1, 3), dtype=torch.float64, device="cuda")
            with torch.no_grad():
                vals.append(float(loss_of(torch, pair_integrals(Vq, C, lists, **SETTINGS), c, w)))
        fd.append((vals[0] - vals[1]) / (2 * h))
    fd = np.array(fd)
    err = np.abs(g[coords] - fd) / np.abs(g).max()
    print("adjoint vs FD (CUDA forward): max rel", err.max())
    assert err.max() <= 1e-6, err.max()


def test_adjoint_matches_oracle_gradient(setup):
    """reference gradient: central FD of the oracle's forward pass (same rules, CPU)"""
    torch, V, C, lists, c, w, coords = setup
    from integrator2_gb300.autograd import pair_integrals
    from oracle import oracle as O
    Vt = torch.tensor(V, dtype=torch.float64, device="cuda", requires_grad=True)
    L = loss_of(torch, pair_integrals(Vt, C, lists, **SETTINGS), c, w)
    L.backward()
    g = Vt.grad.detach().cpu().numpy().reshape(-1)

    def oracle_loss(Vx):
        tot = 0.0
        with O.potential_rule(10, 8, 3, adaptive=0, self_n=0):
            for cls, (pr, ck) in enumerate(zip(lists, c)):
                _, J, P, _ = O.integrate(cls, pr, Vx, C, mode=O.FIXED, level=1)
                tot += float(np.sum(ck * (P + J @ w)))
        return tot

    h = 1e-6
    for k in coords[:8]:
        Vp, Vm = V.copy().reshape(-1), V.copy().reshape(-1)
        Vp[k] += h
        Vm[k] -= h
        fd = (oracle_loss(Vp.reshape(-1, 3)) - oracle_loss(Vm.reshape(-1, 3))) / (2 * h)
        assert abs(g[k] - fd) <= 1e-6 * np.abs(g).max(), (k, g[k], fd)


def local_fd(torch, V, C, lists, c, w, k, h, groups=None, **settings):
    """central difference of L with respect to coordinate k over the pairs that touch its vertex's
    cells: no other pair depends on that coordinate, so this equals the difference of the whole
    loss (without its cancellation).  groups: per class, an array of refinement levels; the
    pairs of each level are then run at that fixed level (the refinement frozen at the levels a
    base run kept)"""
    from integrator2_gb300.autograd import pair_integrals
    cells = np.where((np.asarray(C) == k // 3).any(axis=1))[0]
    sel = [np.isin(l[:, 0], cells) | np.isin(l[:, 1], cells) for l in lists]
    runs = []
    if groups is None:
        runs.append(([l[m] for l, m in zip(lists, sel)], [ck[m] for ck, m in zip(c, sel)], settings))
    else:
        for L in sorted({int(x) for g, m in zip(groups, sel) for x in np.asarray(g)[m]}):
            ms = [m & (np.asarray(g) == L) for g, m in zip(groups, sel)]
            runs.append(([l[m] for l, m in zip(lists, ms)], [ck[m] for ck, m in zip(c, ms)],
                         dict(settings, mode="fixed", level=max(L, 0))))
    vals = []
    for sgn in (1.0, -1.0):
        Vp = V.copy().reshape(-1)
        Vp[k] += sgn * h
        Vq = torch.tensor(Vp.reshape(-1, 3), dtype=torch.float64, device="cuda")
        tot = 0.0
        with torch.no_grad():
            for sub, cs, kw in runs:
                tot += float(loss_of(torch, pair_integrals(Vq, C, sub, **kw), cs, w))
        vals.append(tot)
    return (vals[0] - vals[1]) / (2 * h)


def test_adjoint_fp32_against_fp64(setup):
    """the FP32 adjoint (after a mixed-precision forward) against the FP64 adjoint"""
    torch, V, C, lists, c, w, coords = setup
    from integrator2_gb300 import api
    from integrator2_gb300.autograd import pair_integrals

    def grad(**kw):
        Vt = torch.tensor(V, dtype=torch.float64, device="cuda", requires_grad=True)
        loss_of(torch, pair_integrals(Vt, C, lists, **kw), c, w).backward()
        return Vt.grad.detach().cpu().numpy()

    g64 = grad(**SETTINGS)
    g32 = grad(mode="fixed", level=1, hard_tol=0.0, precision=api.PRECISION_MIXED)
    e32 = np.abs(g32 - g64).max() / np.abs(g64).max()
    print("FP32 adjoint vs FP64 adjoint: max rel", e32)
    assert e32 < 1e-6


def test_adjoint_of_adaptive_run_matches_frozen_finite_differences(setup):
    """relative error control (levels chosen per pair) with the tiered potential and the adaptive
    rule of hard adjacent pairs: the adjoint (refinement frozen at the levels the forward kept,
    potential decisions taken on the values) against central differences with each pair held at
    the level the base run kept; h = 1e-6, bar 1e-6 x max |gradient|"""
    torch, V, C, lists, c, w, coords = setup
    from integrator2_gb300 import api
    from integrator2_gb300.autograd import pair_integrals
    kw = dict(mode="relative", tol=1e-6, max_level=5, hard_tol=1e-8)
    Vt = torch.tensor(V, dtype=torch.float64, device="cuda", requires_grad=True)
    loss_of(torch, pair_integrals(Vt, C, lists, **kw), c, w).backward()
    g = Vt.grad.detach().cpu().numpy().reshape(-1)
    m = api.Mesh3D()
    m.setGeometry(V, C)
    m.prepareMesh(3.0)
    it = api.NumericalIntegrator3D(m, api.qf3D13)
    it.setErrorControl(api.RELATIVE_ERROR_CONTROL, 1e-6, 5)
    it.setHardPairTolerance(1e-8)
    ev = api.EvaluatorJ3DK(m, it)
    levels = []
    for cls, pr in enumerate(lists):
        ev.runClass(cls, pr)
        levels.append(ev.getLevels(cls) if cls != 3 else np.zeros(len(pr), int))
    assert max(int(l.max()) for l in levels[:3]) >= 2  # the run does refine
    err = max(abs(local_fd(torch, V, C, lists, c, w, int(k), 1e-6, groups=levels, hard_tol=1e-8) - g[k]) for k in coords)
    print("adaptive-run adjoint vs frozen FD: max rel", err / np.abs(g).max())
    assert err <= 1e-6 * np.abs(g).max()


@pytest.mark.parametrize("precision", ["fp64", "fp32"])
def test_adjoint_c4_two_hundred_coordinates(precision):
    """C4: 5,120-triangle sphere with a spherical-harmonic radial displacement (degree <= 6,
    coefficients ~ N(0, 0.05^2), seed 4), all four classes (near < 3h), fixed level 1: the FP64 and
    the FP32 adjoint against central differences (h = 1e-6) of the FP64 forward on 200 seeded
    coordinates, bar 1e-6 x max |gradient|"""
    torch = pytest.importorskip("torch")
    ensure_built()
    from integrator2_gb300 import api, meshes, pairs as P
    from integrator2_gb300.autograd import pair_integrals
    V, C = meshes.sh_displaced_icosphere(4, 6, 0.05, 4)
    pl = P.build_pairs(V, C)
    lists = [pl.vertex, pl.edge, pl.far, pl.self_]
    rng = np.random.default_rng(11)
    c = [rng.standard_normal(len(l)) for l in lists]
    w = rng.standard_normal(3)
    prec = api.PRECISION_FP64 if precision == "fp64" else api.PRECISION_MIXED
    Vt = torch.tensor(V, dtype=torch.float64, device="cuda", requires_grad=True)
    loss_of(torch, pair_integrals(Vt, C, lists, precision=prec, **SETTINGS), c, w).backward()
    g = Vt.grad.detach().cpu().numpy().reshape(-1)
    coords = rng.choice(V.size, 200, replace=False)
    err = np.array([abs(local_fd(torch, V, C, lists, c, w, int(k), 1e-6, **SETTINGS) - g[k]) for k in coords]) / np.abs(g).max()
    print(f"C4 {precision} adjoint vs FD on 200 coordinates: max {err.max():.2e}")
    assert err.max() <= 1e-6
