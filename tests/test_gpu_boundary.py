"""The drop-in boundary's remaining reference objects through the C ABI, against the oracle: the SolverTypeTag
names and what each runs, DifferentiableFunctionFactory::op with derivative(f), NewtonRaphson::residual() /
jacobian() / updateFunction(), the assembled scalar, constraintsBelow / createFullVector / createReducedVector,
the AssemblerManipulator matrix hook (springs), NonLinearSolverLogger and ControlLogger, and the bounded device
wait of the persistent CG running out (the timeout status, after which the handle solves normally)."""
import json
import os
import re

import numpy as np
import pytest

import oracle
from ikarus_gb300 import problems

pytestmark = pytest.mark.gpu
sp = pytest.importorskip("scipy.sparse")
GOLD = json.load(open(os.path.join(os.path.dirname(__file__), "golden", "reference_goldens.json")))
FP64_RTOL = 1e-12


def rel_err(a, b):
    return float(np.abs(np.asarray(a) - np.asarray(b)).max() / max(np.abs(b).max(), 1e-300))


def small(seed=3):
    return problems.cantilever(6, 3, 2, L=4.0, jitter=0.15, seed=seed)


def test_solver_type_tags_keep_the_reference_order(ikr):
    names = ["none", "si_ConjugateGradient", "si_LeastSquaresConjugateGradient", "si_BiCGSTAB", "sd_SimplicialLLT",
             "sd_SimplicialLDLT", "sd_SparseLU", "sd_SparseQR", "sd_CholmodSupernodalLLT", "sd_UmfPackLU",
             "sd_SuperLU", "d_PartialPivLU", "d_FullPivLU", "d_HouseholderQR", "d_ColPivHouseholderQR",
             "d_FullPivHouseholderQR", "d_CompleteOrthogonalDecomposition", "d_LLT", "d_LDLT"]
    assert [ikr.SolverTypeTag(i).name for i in range(19)] == names  # linearsolver.hh:28-31
    with pytest.raises(ikr.IkarusError, match="NOT_IMPLEMENTED"):
        ikr.LinearSolver(ikr.SolverTypeTag.sd_SuperLU)  # linearsolver.cpp:51-53 throws


def test_every_sparse_tag_solves_and_dense_tags_reject_the_sparse_tangent(ikr):
    p = small()
    fes, asm = problems.build_gpu(p)
    u = 0.01 * np.random.default_rng(1).standard_normal(p.n_dofs) * (1 - p.fixed)
    req = ikr.FERequirements(fes, u, 0.3)
    K = asm.matrix(req, dbc=ikr.DBCOption.Full)
    b = np.random.default_rng(2).standard_normal(p.n_dofs) * (1 - p.fixed)
    T = ikr.SolverTypeTag
    for tag in (T.si_ConjugateGradient, T.si_LeastSquaresConjugateGradient, T.si_BiCGSTAB):
        ls = ikr.LinearSolver(tag, rtol=1e-12)
        ls.compute(asm)
        x = ls.solve(asm, b)
        assert np.linalg.norm(K @ x - b) <= 1e-11 * np.linalg.norm(b), tag
    for tag in (T.sd_SimplicialLLT, T.sd_SimplicialLDLT, T.sd_SparseLU, T.sd_SparseQR, T.sd_CholmodSupernodalLLT,
                T.sd_UmfPackLU):
        ls = ikr.LinearSolver(tag)  # direct-accuracy solve: 1e-13 whatever is asked of it
        ls.compute(asm)
        x = ls.solve(asm, b)
        it, rel = ls.last_info()
        assert rel <= ikr.DIRECT_SOLVE_RTOL, (tag, rel)
        assert np.linalg.norm(K @ x - b) <= 1e-12 * np.linalg.norm(b), tag
    for tag in range(int(T.d_PartialPivLU), int(T.d_LDLT) + 1):
        ls = ikr.LinearSolver(T(tag))
        with pytest.raises(ikr.IkarusError, match="NOT_IMPLEMENTED"):
            ls.compute(asm)
    with pytest.raises(ikr.IkarusError, match="INVALID_STATE"):
        ikr.LinearSolver(T.none).compute(asm)
    fes32, asm32 = problems.build_gpu(p, precision=1)
    asm32.matrix(ikr.FERequirements(fes32, u, 0.3), dbc=ikr.DBCOption.Full, export=False)
    with pytest.raises(ikr.IkarusError, match="NOT_IMPLEMENTED"):  # needs the FP64 outer solve
        ikr.LinearSolver(T.sd_SimplicialLDLT).compute(asm32)


@pytest.mark.parametrize("tag", ["sd_SimplicialLDLT", "sd_UmfPackLU"])
def test_direct_tags_reproduce_the_cantilever_goldens(ikr, tag):
    """tests/src/testcantileverbeamEAS.cpp:60-124 with the reference's own solver tags (UmfPackLU there, the
    SimplicialLDLT default elsewhere) and the Newton's default linear tolerance."""
    g = GOLD["cantilever_3d"]
    want = g["results"]["GreenLagrangeStrain"]["NeoHooke"]
    p = problems.cantilever_golden(1, g["eas_parameters"]["GreenLagrangeStrain"])
    fes, asm = problems.build_gpu(p)
    req = ikr.FERequirements(fes)
    ls = ikr.LinearSolver(ikr.SolverTypeTag[tag])
    nr = ikr.NewtonRaphson(asm, ikr.NewtonRaphsonConfig(ikr.NRSettings(tol=g["tol"]), ls))
    info = ikr.LoadControl(nr, g["load_steps"], (0.0, 1.0)).run(req)
    assert info.success and info.totalIterations == want["iterations"]
    assert abs(np.abs(req.globalSolution()).max() - want["max_disp"]) <= 1e-10 * want["max_disp"]


def test_nonlinear_operator_and_its_derivatives_match_oracle(ikr):
    p = small()
    fes, asm = problems.build_gpu(p)
    o = oracle.from_problem(p)
    u = 0.01 * np.random.default_rng(5).standard_normal(p.n_dofs) * (1 - p.fixed)
    req = ikr.FERequirements(fes, u, 0.4)
    energy = sum(o.element_energy(e, u, 0.4) for e in range(p.mesh.n_elems))
    # energy -> forces -> stiffness (AffordanceCollections::elastoStatics)
    f = ikr.DifferentiableFunctionFactory.op(asm, ikr.AffordanceCollections.elastoStatics)
    assert rel_err(f(req), energy) <= FP64_RTOL
    assert rel_err(asm.scalar(req), energy) <= FP64_RTOL
    df = ikr.derivative(f)
    assert rel_err(df(req), o.assemble_vector(u, 0.4)) <= FP64_RTOL
    K = ikr.derivative(df)(req)
    assert rel_err(K.toarray(), o.assemble_matrix_dense(u, 0.4)) <= FP64_RTOL
    with pytest.raises(ikr.IkarusError, match="ARG"):
        ikr.derivative(ikr.derivative(df))(req)
    # forces -> stiffness, Reduced option
    g = ikr.DifferentiableFunctionFactory.op(asm, ikr.AffordanceCollection(), ikr.DBCOption.Reduced)
    assert rel_err(g(req), o.assemble_vector(u, 0.4, oracle.DBC_REDUCED)) <= FP64_RTOL
    Kr = ikr.derivative(g)(req)
    assert rel_err(Kr.toarray(), o.assemble_matrix_dense(u, 0.4, oracle.DBC_REDUCED)) <= FP64_RTOL
    # EAS elements have no potential (enhancedassumedstrains.hh:305-309)
    pe = problems.cantilever(4, 2, 2, eas=1, n_eas=9)
    fe2, asm2 = problems.build_gpu(pe)
    fe_op = ikr.DifferentiableFunctionFactory.op(asm2, ikr.AffordanceCollections.elastoStatics)
    with pytest.raises(ikr.IkarusError, match="NOT_IMPLEMENTED"):
        fe_op(ikr.FERequirements(fe2))


def test_newton_residual_jacobian_and_update_function(ikr):
    p = small()
    fes, asm = problems.build_gpu(p)
    o = oracle.from_problem(p)
    nr = ikr.NewtonRaphson(asm, ikr.NewtonRaphsonConfig(ikr.NRSettings(), ikr.LinearSolver()))
    u = 0.01 * np.random.default_rng(6).standard_normal(p.n_dofs) * (1 - p.fixed)
    req = ikr.FERequirements(fes, u, 0.5)
    assert rel_err(nr.residual()(req), o.assemble_vector(u, 0.5)) <= FP64_RTOL
    assert rel_err(nr.jacobian()(req).toarray(), o.assemble_matrix_dense(u, 0.5)) <= FP64_RTOL
    dx = 1e-3 * np.random.default_rng(7).standard_normal(p.n_dofs)
    nr.updateFunction()(req, dx)
    assert np.array_equal(req.globalSolution(), u + dx)


def test_constraints_below_and_reduced_full_vectors_match_oracle(ikr):
    p = small()
    fes, asm = problems.build_gpu(p)
    o = oracle.from_problem(p)
    assert np.array_equal(asm.constraintsBelow(), o.constraints_below())
    assert asm.reducedSize() == o.reduced_size()
    u = 0.01 * np.random.default_rng(8).standard_normal(p.n_dofs) * (1 - p.fixed)
    Rf = o.assemble_vector(u, 0.2, oracle.DBC_FULL)
    Rr = o.assemble_vector(u, 0.2, oracle.DBC_REDUCED)
    assert np.array_equal(asm.createReducedVector(Rf), Rr)
    assert np.array_equal(asm.createFullVector(Rr), Rf)  # constrained entries zero in both


def test_manipulator_matrix_entries_add_springs_after_the_dirichlet_treatment(ikr):
    """testassembler.cpp:212-219: springs on the diagonal (and here one off-diagonal coupling) after assembly."""
    p = small()
    fes, asm = problems.build_gpu(p)
    o = oracle.from_problem(p)
    u = 0.01 * np.random.default_rng(9).standard_normal(p.n_dofs) * (1 - p.fixed)
    tip = 3 * (p.mesh.n_nodes - 1)
    rows, cols, vals = [tip + 1, tip + 2, tip + 1, 0], [tip + 1, tip + 2, tip + 2, 0], [596482.0, 596482.0, 7.5, 3.0]
    asm.add_matrix_entries(rows, cols, vals)
    req = ikr.FERequirements(fes, u, 0.1)
    for dbc, odbc in [(ikr.DBCOption.Full, oracle.DBC_FULL), (ikr.DBCOption.Raw, oracle.DBC_RAW)]:
        K = asm.matrix(req, dbc=dbc).toarray()
        Ko = o.assemble_matrix_dense(u, 0.1, odbc)
        for r, c, v in zip(rows, cols, vals):
            Ko[r, c] += v  # dof 0 is constrained: the Full option's unit diagonal becomes 1 + 3
        assert rel_err(K, Ko) <= FP64_RTOL, dbc
    Kr = asm.matrix(req, dbc=ikr.DBCOption.Reduced).toarray()
    free = np.nonzero(p.fixed == 0)[0]
    Ko = o.assemble_matrix_dense(u, 0.1, oracle.DBC_RAW)
    for r, c, v in zip(rows, cols, vals):
        Ko[r, c] += v
    assert rel_err(Kr, Ko[np.ix_(free, free)]) <= FP64_RTOL
    with pytest.raises(ikr.IkarusError, match="ARG"):
        asm.add_matrix_entries([0], [3 * (p.mesh.n_nodes - 1)], [1.0])  # not in the pattern


def test_loggers_print_the_reference_lines(ikr):
    p = problems.config1()
    p.load_steps = 3
    ref = oracle.from_problem(p).load_control(3, tol=p.tol)
    fes, asm = problems.build_gpu(p)
    req = ikr.FERequirements(fes)
    nr = ikr.NewtonRaphson(asm, ikr.NewtonRaphsonConfig(ikr.NRSettings(tol=p.tol, linear_rtol=1e-12),
                                                         ikr.LinearSolver(rtol=1e-12)))
    nlog = ikr.NonLinearSolverLogger(sink=lambda line: None).subscribeTo(nr)
    lc = ikr.LoadControl(nr, 3)
    clog = ikr.ControlLogger(sink=lambda line: None).subscribeTo(lc)
    info = lc.run(req)
    assert info.success
    L = nlog.lines
    assert L.count("Non-linear solver started:") == 4  # the initial equilibrium solve and three load steps
    assert L[1].split() == ["Ite", "normR", "normD", "lambda"]
    its = [int(m.group(1)) for m in map(re.compile(r"^Number of iterations: (\d+)$").match, L) if m]
    assert its == list(ref["iterations"])  # the initial solve at lambda = 0 finishes with 0 iterations
    rows = [line.split() for line in L if re.match(r"^ \d", line)]
    assert len(rows) == sum(ref["iterations"])
    assert float(rows[-1][3]) == pytest.approx(1.0, rel=1e-2)  # lambda column after the last step
    C = clog.lines
    assert C[1] == "Started Load Control Method" and C[-3] == "End of Load Control Method"
    assert C[-2] == f"Total number of iterations: {sum(ref['iterations']):3d}"
    steps = [line for line in C if line.startswith("Load step:")]
    assert [int(s.split()[2]) for s in steps] == [-1, 0, 1, 2]
    assert steps[0].endswith("Step size =  0.00e+00") and steps[1].endswith("Step size =  3.33e-01")
    assert re.match(r"^Elapsed time: \d+ ms$", C[-1])


def test_bounded_grid_barrier_wait_runs_out_and_the_handle_recovers(ikr):
    """The persistent CG's grid-barrier waits are bounded: with CTA 0 withholding its first arrival (a test switch
    of one launch) every CTA's wait runs out after the configured polls, the solve reports IKR_ERR_TIMEOUT, and the
    same handles then solve to the same result as a fresh solver."""
    p = problems.cantilever(16, 4, 4, jitter=0.1, seed=1)
    fes, asm = problems.build_gpu(p, precision=1)
    asm.matrix(ikr.FERequirements(fes), dbc=ikr.DBCOption.Full, export=False)
    b = np.random.default_rng(3).standard_normal(p.n_dofs) * (1 - p.fixed)
    ref = ikr.LinearSolver(rtol=1e-5)
    ref.set_kernel(spmv_kind=9, l2_keep_fraction=0.0)  # a persistent kind
    ref.compute(asm)
    x_ref = ref.solve(asm, b)
    ls = ikr.LinearSolver(rtol=1e-5)
    ls.set_kernel(spmv_kind=9, l2_keep_fraction=0.0)
    ls.compute(asm)
    assert ls.kernel_info()[0] == 9
    ls.set_wait_test(barrier_polls=4096, withhold_first_arrival=True)
    with pytest.raises(ikr.IkarusError, match="TIMEOUT"):
        ls.solve(asm, b)
    x = ls.solve(asm, b)  # the switch acted on one launch; the context and the handles stay usable
    assert np.array_equal(x, x_ref)
