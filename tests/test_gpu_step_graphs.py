"""Newton iterations as CUDA graphs: with NRSettings.step_graphs (the default) every Newton iteration after the
first of a solver's life runs as one graph launch (tangent, block-Jacobi inverse, persistent CG, update, residual,
norms).  The iterates, norms and iteration counts are bit-identical to the launch-by-launch iteration, in the plain
FP64 and the mixed form, with the lambda-linear traction, point loads and a function-defined load (whose host
evaluation happens before each launch), and the graph path really ran."""
import numpy as np
import pytest

from ikarus_gb300 import problems

pytestmark = pytest.mark.gpu


def run(ikr, p, precision, graphs, body=None):
    fes, asm = problems.build_gpu(p, precision=precision)
    if body is not None:
        fes.add_volume_load(body)
    ls = ikr.LinearSolver()
    ls.set_kernel(spmv_kind=9, l2_keep_fraction=0.0)  # a persistent CG kind
    if precision:
        st = ikr.NRSettings(tol=1e-8, maxIter=40, relative=True, eisenstat_walker=True, linear_rtol=2e-2,
                            linear_rtol_min=1e-5, step_graphs=graphs)
    else:
        st = ikr.NRSettings(tol=1e-9, maxIter=40, relative=True, linear_rtol=1e-11, step_graphs=graphs)
    nr = ikr.NewtonRaphson(asm, ikr.NewtonRaphsonConfig(st, ls))
    norms = []
    nr.subscribe(lambda m, s: norms.append((int(m), s["residualNorm"], s["correctionNorm"])))
    req = ikr.FERequirements(fes)
    info = ikr.LoadControl(nr, p.load_steps).run(req)
    assert info.success
    return req.globalSolution(), [s.iterations for s in info.solverInfos], norms, nr.graph_iterations()


@pytest.mark.parametrize("precision", [0, 1])
def test_graph_iterations_are_bit_identical_to_launch_by_launch(ikr, precision):
    p = problems.cantilever(24, 6, 6, jitter=0.1, seed=5, load_steps=4)
    p.pl_dofs = np.array([3 * (p.mesh.n_nodes - 1) + 1], dtype=np.int32)
    p.pl_values = np.array([0.05])

    def body(X, lam):
        return np.stack([0.0 * X[:, 0], 0.0 * X[:, 0], -0.1 * lam ** 2 + 0.0 * X[:, 0]], axis=1)

    u0, it0, n0, g0 = run(ikr, p, precision, False, body)
    u1, it1, n1, g1 = run(ikr, p, precision, True, body)
    assert g0 == 0 and g1 > 0
    assert it1 == it0
    assert n1 == n0  # every observer message with its norms, in the same order
    assert np.array_equal(u1, u0)
