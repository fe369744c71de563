"""Mixed-precision form (FP32 bulk, FP64 singular parts / estimator / hard pairs) through the
C-ABI: per class and per channel error against the FP64 form and against the oracle's
high-order answer."""
import numpy as np
import pytest

from tests._util import ensure_built, rel_rows

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def api():
    ensure_built()
    from integrator2_gb300 import api as A
    return A


def _run(api, V, C, cls, pairs, precision, mode="relative", level=0):
    m = api.Mesh3D()
    m.setGeometry(V, C)
    m.prepareMesh(3.0)
    it = api.NumericalIntegrator3D(m, api.qf3D13)
    if mode == "relative":
        it.setErrorControl(api.RELATIVE_ERROR_CONTROL, 1e-6, 5)
    else:
        it.setFixedRefinementLevel(level)
    it.setPrecision(precision)
    ev = api.EvaluatorJ3DK(m, it)
    ev.runClass(cls, pairs)
    return ev.getResults(cls), ev.getPotentials(cls), ev.getLevels(cls)


def test_mixed_matches_fp64_at_fixed_level(api):
    """same rule, same refinement: the difference is the FP32 rounding of the bulk.  FP32
    rounding acts like a relative input perturbation of a few 1e-8, so the per-pair bar grows
    with kappa, the pair's measured relative sensitivity to such perturbations:
    max(1e-5, 1e-7 kappa); the rms over the class stays below 1e-6."""
    from integrator2_gb300 import meshes, pairs as P
    from oracle import oracle as O
    V, C = meshes.jittered_icosphere(3, 0.15, 11)
    pl = P.build_pairs(V, C)
    worst = {}
    for cls in (0, 1, 2, 3):
        pr = pl.by_class(cls)[::3]
        J64, P64, _ = _run(api, V, C, cls, pr, api.PRECISION_FP64, "fixed", 1)
        J32, P32, _ = _run(api, V, C, cls, pr, api.PRECISION_MIXED, "fixed", 1)
        eJ = rel_rows(J32, J64) if cls != 3 else np.abs(J32 - J64).max(axis=1)
        eP = np.abs(P32 - P64) / np.abs(P64)
        kap = O.conditioning(cls, pr, V, C, 1) if cls != 3 else np.ones(len(pr))
        bar = np.maximum(1e-5, 1e-7 * kap)
        w = int(np.argmax(eJ / bar))
        worst[cls] = (float(eJ.max()), float(eP.max()), float(np.sqrt(np.mean(eJ ** 2))), float(kap[w]), pr[w].tolist())
        assert np.all(eJ <= bar) and eP.max() < 1e-5, (cls, worst[cls])
        assert np.sqrt(np.mean(eJ ** 2)) < 1e-6 and np.sqrt(np.mean(eP ** 2)) < 1e-6, (cls, worst[cls])
    print("mixed vs fp64 (J max, P max, J rms, kappa and pair of the worst):", worst)


def test_mixed_accuracy_against_high_order(api):
    from integrator2_gb300 import meshes, pairs as P
    from oracle import oracle as O
    V, C = meshes.jittered_icosphere(3, 0.15, 12)
    pl = P.build_pairs(V, C)
    rng = np.random.default_rng(0)
    report = {}
    for cls in (0, 1, 2):
        pr = pl.by_class(cls)
        pr = pr[np.sort(rng.choice(len(pr), min(300, len(pr)), replace=False))]
        J, Pm, _ = _run(api, V, C, cls, pr, api.PRECISION_MIXED)
        with O.potential_rule(40, 32, 3, adaptive=1e-10, depth=18, every_pair=True):
            _, oJ, oP, _ = O.integrate(cls, pr, V, C, mode=O.FIXED, level=4)
        eJ = rel_rows(J, oJ)
        eP = np.abs(Pm - oP) / np.abs(oP)
        report[cls] = (float(eJ.max()), float(eP.max()))
        assert eJ.max() < 1e-5 and eP.max() < 1e-5, (cls, report[cls])
    print("mixed vs high-order oracle (J max, P max):", report)
