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


def test_adjoint_fp32_and_adaptive(setup):
    """the FP32 adjoint (after a mixed-precision forward) against the FP64 adjoint, and the
    adjoint of an adaptive run (refinement frozen at the levels the forward kept) against the
    fixed-level adjoint at the deepest level reached"""
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
    assert e32 < 1e-4
    ga = grad(mode="relative", tol=1e-6, max_level=5, hard_tol=1e-8)
    assert np.isfinite(ga).all()
    assert np.abs(ga - g64).max() / np.abs(g64).max() < 1e-3
