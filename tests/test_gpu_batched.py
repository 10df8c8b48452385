"""Independent instances solved together (one CG launch per Newton iteration, CTA per instance) against the
oracle solving each instance on its own."""
import numpy as np
import pytest

import oracle
from ikarus_gb300 import problems

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("precision", [0, 1])
def test_batched_instances_match_individual_oracle_solves(ikr, precision, parity_log):
    """Plain FP64: every instance's Newton to ||R|| <= 1e-9 ||R0|| per step (1e-10 is at the FP64 residual floor of
    one of these small beams), displacement within 1e-8 of the oracle's (solved to the same tolerance with its
    direct solve).  Mixed: FP32 tangent and CG with the FP64
    residual test at 1e-8 per step (the benchmark's criterion); its displacement error against the oracle is
    logged and bounded by 1e-8 as well."""
    bp = problems.batched_cantilevers(n=12, seed=3, nx=(3, 8), nyz=(1, 3), E=(1e3, 1e4), t=(0.1, 0.5),
                                      load_steps=4)
    fes, asm = problems.build_gpu_batched(bp, precision=precision)
    req = ikr.FERequirements(fes)
    if precision == 0:
        st = ikr.NRSettings(tol=1e-9, maxIter=30, relative=True, linear_rtol=1e-12)
    else:
        st = ikr.NRSettings(tol=1e-8, maxIter=30, relative=True, eisenstat_walker=True, linear_rtol=1e-2,
                            linear_rtol_min=1e-6)
    nr = ikr.NewtonRaphson(asm, ikr.NewtonRaphsonConfig(st, ikr.LinearSolver(ikr.SolverTypeTag.gpu_PCG_Batched)))
    info = ikr.LoadControl(nr, bp.load_steps).run(req)
    assert info.success
    its, rn, conv = nr.instance_info()
    assert (conv == 1).all()
    u = req.globalSolution()
    worst = 0.0
    for i, part in enumerate(bp.parts):
        ref = oracle.from_problem(part).load_control(bp.load_steps, tol=1e-9, tol_mode=1, max_iter=30)
        ui = u[3 * bp.node_offsets[i]:3 * bp.node_offsets[i + 1]]
        worst = max(worst, np.abs(ui - ref["u"]).max() / np.abs(ref["u"]).max())
    form = "FP64" if precision == 0 else "mixed"
    assert parity_log(f"batched {form}: max over instances of max|u - u_oracle| / max|u_oracle|", worst,
                      1e-8)


def test_an_inverting_instance_is_taken_out_and_the_others_converge(ikr):
    """The reference aborts on det C <= 0 (materialhelpers.hh:119-126); in a batched solve the instance whose
    elements invert is taken out (status -1) and every other instance still converges to the oracle's path."""
    bp = problems.batched_cantilevers(n=6, seed=5, nx=(3, 6), nyz=(1, 2), E=(1e3, 1e3), t=(0.2, 0.3), load_steps=3)
    bad = 2
    sel = (bp.face_elem >= bp.elem_offsets[bad]) & (bp.face_elem < bp.elem_offsets[bad + 1])
    bp.face_traction[sel] *= 1e4
    fes, asm = problems.build_gpu_batched(bp, precision=1)
    req = ikr.FERequirements(fes)
    st = ikr.NRSettings(tol=1e-8, maxIter=30, relative=True, eisenstat_walker=True, linear_rtol=1e-2,
                        linear_rtol_min=1e-6)
    nr = ikr.NewtonRaphson(asm, ikr.NewtonRaphsonConfig(st, ikr.LinearSolver(ikr.SolverTypeTag.gpu_PCG_Batched)))
    info = ikr.LoadControl(nr, bp.load_steps).run(req)
    assert info.success
    _, _, conv = nr.instance_info()
    assert conv[bad] == -1 and (np.delete(conv, bad) == 1).all()
    u = req.globalSolution()
    for i, part in enumerate(bp.parts):
        if i == bad:
            continue
        ref = oracle.from_problem(part).load_control(bp.load_steps, tol=1e-8, tol_mode=1)
        ui = u[3 * bp.node_offsets[i]:3 * bp.node_offsets[i + 1]]
        assert np.abs(ui - ref["u"]).max() <= 1e-6 * np.abs(ref["u"]).max(), i


def test_excluded_instances_take_no_part_and_the_others_are_unchanged(ikr):
    """ikr_newton_exclude_instances: the excluded instances get no corrections (their displacement stays zero,
    status -3); the others reach the same solution as without the exclusion (within the FP64 rounding of a
    different CTA plan), and a following run of only the excluded instances solves them as well -- the FP64 retry
    the benchmark applies to the instances an FP32 run took out."""
    bp = problems.batched_cantilevers(n=8, seed=3, nx=(3, 8), nyz=(1, 3), E=(1e3, 1e4), t=(0.1, 0.5), load_steps=3)
    st = ikr.NRSettings(tol=1e-9, maxIter=30, relative=True, linear_rtol=1e-12)

    def run(exclude=None):
        fes, asm = problems.build_gpu_batched(bp, precision=0)
        req = ikr.FERequirements(fes)
        nr = ikr.NewtonRaphson(asm, ikr.NewtonRaphsonConfig(st, ikr.LinearSolver(ikr.SolverTypeTag.gpu_PCG_Batched)))
        if exclude is not None:
            nr.exclude_instances(exclude)
        info = ikr.LoadControl(nr, bp.load_steps).run(req)
        return info, nr.instance_info()[2], req.globalSolution()

    info0, conv0, u0 = run()
    assert info0.success and (conv0 == 1).all()
    mask = np.zeros(8, dtype=bool)
    mask[[1, 6]] = True
    info1, conv1, u1 = run(mask)
    assert info1.success
    assert (conv1[mask] == -3).all() and (conv1[~mask] == 1).all()
    info2, conv2, u2 = run(~mask)
    assert info2.success and (conv2[mask] == 1).all() and (conv2[~mask] == -3).all()
    for i in range(8):
        sl = slice(3 * bp.node_offsets[i], 3 * bp.node_offsets[i + 1])
        scale = np.abs(u0[sl]).max()
        if mask[i]:
            assert not u1[sl].any()
            assert np.abs(u2[sl] - u0[sl]).max() <= 1e-9 * scale
        else:
            assert not u2[sl].any()
            assert np.abs(u1[sl] - u0[sl]).max() <= 1e-9 * scale
    with pytest.raises(ikr.IkarusError):
        fes, asm = problems.build_gpu_batched(bp, precision=0)
        nr = ikr.NewtonRaphson(asm, ikr.NewtonRaphsonConfig(st, ikr.LinearSolver(ikr.SolverTypeTag.gpu_PCG_Batched)))
        nr.exclude_instances(np.zeros(5, dtype=bool))


def test_batched_solve_notifies_observers_and_counts_cg_iterations_per_instance(ikr):
    """The batched Newton notifies INIT, ITERATION_STARTED/ENDED and FINISHED like the single-system one
    (newtonraphson.hh:193-257), with the largest residual norm over the instances in the solve; the per-instance
    CG iteration counts sum to the solve's linear iterations."""
    bp = problems.batched_cantilevers(n=5, seed=3, nx=(3, 6), nyz=(1, 2), E=(1e3, 1e4), t=(0.1, 0.4), load_steps=2)
    fes, asm = problems.build_gpu_batched(bp, precision=1)
    st = ikr.NRSettings(tol=1e-8, maxIter=30, relative=True, eisenstat_walker=True, linear_rtol=1e-2,
                        linear_rtol_min=1e-6)
    nr = ikr.NewtonRaphson(asm, ikr.NewtonRaphsonConfig(st, ikr.LinearSolver(ikr.SolverTypeTag.gpu_PCG_Batched)))
    M = ikr.NonLinearSolverMessages
    seen = []
    nr.subscribe(lambda msg, s: seen.append((msg, s["iterations"], s["residualNorm"])))
    req = ikr.FERequirements(fes)
    req.insertParameter(0.5)
    info = nr.solve(req)
    assert info.success
    msgs = [m for m, _, _ in seen]
    assert msgs[0] == M.INIT and msgs[-1] == M.FINISHED_SUCESSFULLY
    ended = [(it, rn) for m, it, rn in seen if m == M.ITERATION_ENDED]
    assert len(ended) == info.iterations == msgs.count(M.ITERATION_STARTED)
    assert [it for it, _ in ended] == list(range(1, info.iterations + 1))
    its, rn, conv = nr.instance_info()
    assert (conv == 1).all()
    assert ended[-1][1] == pytest.approx(rn.max(), rel=0, abs=0)
    lin = nr.instance_linear_iterations()
    assert lin.sum() == info.linearIterations and (lin > 0).all()


_CHUNK_REF = {}


@pytest.mark.parametrize("precision", [0, 1])
@pytest.mark.parametrize("variant,first_chunk", [(-1, 0), (0, 0), (1, 0), (2, 0), (3, 0), (4, 0), (5, 0), (-1, 3),
                                                   (0, 5), (1, 1), (2, 4), (3, 2), (4, 3), (5, 2)])
def test_chunked_cg_launches_of_every_variant_match_the_oracle(ikr, precision, variant, first_chunk, parity_log):
    """The batched CG continues each instance's PCG across launches of a few iterations, re-planned over the
    instances still running (first_chunk 1..5: every solve spans many launches); every kernel variant (0 row loop,
    1 one row per thread, 2 / 3 / 5 four / eight / sixteen threads per row with the matrix in shared memory, 4 one
    instance per thread-block cluster -- FP32; FP64 runs fall back to the row loop --, -1 the planner's choice) gives converged displacements that match the oracle's solves (FP64 1e-8 at ||R|| <= 1e-9 ||R0||; mixed
    1e-8 at 1e-8)."""
    bp = problems.batched_cantilevers(n=7, seed=11, nx=(3, 9), nyz=(1, 3), E=(1e3, 1e4), t=(0.1, 0.5), load_steps=3)
    fes, asm = problems.build_gpu_batched(bp, precision=precision)
    req = ikr.FERequirements(fes)
    if precision == 0:
        st = ikr.NRSettings(tol=1e-9, maxIter=30, relative=True, linear_rtol=1e-12)
    else:
        st = ikr.NRSettings(tol=1e-8, maxIter=30, relative=True, eisenstat_walker=True, linear_rtol=1e-2,
                            linear_rtol_min=1e-6)
    nr = ikr.NewtonRaphson(asm, ikr.NewtonRaphsonConfig(st, ikr.LinearSolver(ikr.SolverTypeTag.gpu_PCG_Batched)))
    nr.set_batched_cg(variant=variant, first_chunk=first_chunk)
    info = ikr.LoadControl(nr, bp.load_steps).run(req)
    assert info.success
    _, _, conv = nr.instance_info()
    assert (conv == 1).all()
    if first_chunk:
        assert nr.batched_cg_launches() > info.totalIterations
    if "u" not in _CHUNK_REF:
        _CHUNK_REF["u"] = [oracle.from_problem(part).load_control(bp.load_steps, tol=1e-9, tol_mode=1,
                                                                   max_iter=30)["u"] for part in bp.parts]
    u = req.globalSolution()
    worst = max(np.abs(u[3 * bp.node_offsets[i]:3 * bp.node_offsets[i + 1]] - ref).max() / np.abs(ref).max()
                for i, ref in enumerate(_CHUNK_REF["u"]))
    form = "FP64" if precision == 0 else "mixed"
    by = nr.batched_cg_variant_launches().tolist()
    assert parity_log(f"batched {form}, variant={variant}, first_chunk={first_chunk} (launches per variant {by}): "
                      "max rel. error vs oracle", worst, 1e-8)


def _escalated_run(ikr, bp, primary_settings, take_out=True, observe=None, concurrent=True):
    fes, asm = problems.build_gpu_batched(bp, precision=1)
    nr = ikr.NewtonRaphson(asm, ikr.NewtonRaphsonConfig(primary_settings,
                                                        ikr.LinearSolver(ikr.SolverTypeTag.gpu_PCG_Batched)))
    nr.set_batched_take_out(take_out)
    fes64, asm64 = problems.build_gpu_batched(bp, precision=0)
    nr64 = ikr.NewtonRaphson(asm64, ikr.NewtonRaphsonConfig(
        ikr.NRSettings(tol=1e-9, maxIter=30, relative=True, linear_rtol=1e-12),
        ikr.LinearSolver(ikr.SolverTypeTag.gpu_PCG_Batched)))
    req64 = ikr.FERequirements(fes64)
    lc = ikr.LoadControl(nr, bp.load_steps)
    lc.set_escalation(nr64, req64)
    lc.set_escalation_concurrent(concurrent)
    if observe:
        lc.subscribe(lambda msg, s: observe(msg, s, lc))
    req = ikr.FERequirements(fes)
    info = lc.run(req)
    _, _, conv = nr.instance_info()
    status = lc.instance_status()
    esc = lc.escalated()
    assert (status[~esc] == conv[~esc]).all()
    conv64 = np.where(esc, status, -3)
    return info, req.globalSolution(), esc, conv, conv64


def test_escalation_solves_in_fp64_what_the_fp32_solver_takes_out(ikr, parity_log):
    """Precision escalation of a batched load control: with a CG capped at 3 iterations every FP32 solve is unsolved
    (status -4) in the first step, so every instance continues with the FP64 solver from the step's start; the
    combined solution matches the oracle's solves (1e-8), and the FP32 solver's statuses say why each escalated."""
    bp = problems.batched_cantilevers(n=5, seed=11, nx=(3, 8), nyz=(1, 3), E=(1e3, 1e4), t=(0.1, 0.5), load_steps=3)
    st = ikr.NRSettings(tol=1e-8, maxIter=30, relative=True, linear_rtol=1e-8, linear_max_iter=3)
    info, u, esc, conv, conv64 = _escalated_run(ikr, bp, st)
    assert info.success
    assert esc.all() and (conv == -4).all() and (conv64 == 1).all()
    worst = 0.0
    for i, part in enumerate(bp.parts):
        ref = oracle.from_problem(part).load_control(bp.load_steps, tol=1e-9, tol_mode=1, max_iter=30)["u"]
        worst = max(worst, np.abs(u[3 * bp.node_offsets[i]:3 * bp.node_offsets[i + 1]] - ref).max()
                    / np.abs(ref).max())
    assert parity_log("batched escalation (all instances to FP64): max rel. error vs oracle", worst, 1e-8)


@pytest.mark.parametrize("concurrent", [True, False])
def test_escalation_mid_run_starts_from_the_step_start(ikr, concurrent, parity_log):
    """An FP32 solver allowed 3 Newton iterations per step takes out the instances that need more in some step;
    each continues in FP64 from the state at the start of that step (the converged state of the step before), and
    the combined load path matches the oracle's (1e-8) for every instance -- with the escalated instances' later
    steps solved on a second thread and stream while the FP32 solver does the step, and one after the other."""
    bp = problems.batched_cantilevers(n=8, seed=5, nx=(3, 8), nyz=(1, 3), E=(1e2, 1e4), t=(0.1, 1.0), load_steps=4)
    st = ikr.NRSettings(tol=1e-8, maxIter=3, relative=True, eisenstat_walker=True, linear_rtol=1e-2,
                        linear_rtol_min=1e-6)
    first_step = {}

    def observe(msg, s, lc):
        if msg == ikr.ControlMessages.STEP_ENDED and s["loadStep"] >= 0:
            for i in np.nonzero(lc.escalated())[0]:
                first_step.setdefault(int(i), s["loadStep"])

    info, u, esc, conv, conv64 = _escalated_run(ikr, bp, st, observe=observe, concurrent=concurrent)
    assert info.success
    assert ((conv == 1) | (esc & (conv64 == 1))).all()
    assert set(np.nonzero(esc)[0].tolist()) == set(first_step)
    worst = 0.0
    for i, part in enumerate(bp.parts):
        ref = oracle.from_problem(part).load_control(bp.load_steps, tol=1e-9, tol_mode=1, max_iter=30)["u"]
        worst = max(worst, np.abs(u[3 * bp.node_offsets[i]:3 * bp.node_offsets[i + 1]] - ref).max()
                    / np.abs(ref).max())
    assert parity_log(f"batched escalation mid-run (concurrent={concurrent}, escalated at steps "
                      f"{sorted(first_step.values())}): max rel. error vs oracle", worst, 1e-8)


def test_escalated_instance_that_inverts_in_fp64_too_is_taken_out(ikr):
    """An instance whose elements invert in both precisions ends taken out by the FP64 solver; the others stay
    with the FP32 solver and converge."""
    bp = problems.batched_cantilevers(n=6, seed=5, nx=(3, 6), nyz=(1, 2), E=(1e3, 1e3), t=(0.2, 0.3), load_steps=3)
    bad = 2
    sel = (bp.face_elem >= bp.elem_offsets[bad]) & (bp.face_elem < bp.elem_offsets[bad + 1])
    bp.face_traction[sel] *= 1e4
    st = ikr.NRSettings(tol=1e-8, maxIter=30, relative=True, eisenstat_walker=True, linear_rtol=1e-2,
                        linear_rtol_min=1e-6)
    info, u, esc, conv, conv64 = _escalated_run(ikr, bp, st)
    assert info.success
    assert esc[bad] and conv64[bad] == -1 and conv[bad] in (-1, -4)
    assert (np.delete(conv, bad) == 1).all() and not np.delete(esc, bad).any()


def test_escalation_without_failures_changes_nothing_and_bad_twins_are_rejected(ikr):
    """With nothing taken out the escalated run is the plain run (same displacement bit for bit, nothing escalated);
    an escalation solver over an element set with other instances, or a requirement of another set, is an ARG
    error."""
    bp = problems.batched_cantilevers(n=4, seed=3, nx=(3, 6), nyz=(1, 2), E=(1e3, 1e4), t=(0.1, 0.3), load_steps=2)
    st = ikr.NRSettings(tol=1e-8, maxIter=30, relative=True, eisenstat_walker=True, linear_rtol=1e-2,
                        linear_rtol_min=1e-6)

    def run(with_escalation):
        fes, asm = problems.build_gpu_batched(bp, precision=1)
        nr = ikr.NewtonRaphson(asm, ikr.NewtonRaphsonConfig(st, ikr.LinearSolver(ikr.SolverTypeTag.gpu_PCG_Batched)))
        lc = ikr.LoadControl(nr, bp.load_steps)
        keep = None
        if with_escalation:
            fes64, asm64 = problems.build_gpu_batched(bp, precision=0)
            nr64 = ikr.NewtonRaphson(asm64, ikr.NewtonRaphsonConfig(
                st, ikr.LinearSolver(ikr.SolverTypeTag.gpu_PCG_Batched)))
            req64 = ikr.FERequirements(fes64)
            lc.set_escalation(nr64, req64)
            keep = (fes64, asm64, nr64, req64)
        req = ikr.FERequirements(fes)
        info = lc.run(req)
        assert info.success
        esc = lc.escalated() if with_escalation else None
        return req.globalSolution(), esc, lc.instance_status() if with_escalation else None, keep

    u0, _, _, _ = run(False)
    u1, esc, status, _ = run(True)
    assert not esc.any() and (status == 1).all()
    assert np.array_equal(u0, u1)

    fes, asm = problems.build_gpu_batched(bp, precision=1)
    nr = ikr.NewtonRaphson(asm, ikr.NewtonRaphsonConfig(st, ikr.LinearSolver(ikr.SolverTypeTag.gpu_PCG_Batched)))
    lc = ikr.LoadControl(nr, bp.load_steps)
    other = problems.batched_cantilevers(n=3, seed=4, nx=(3, 6), nyz=(1, 2), load_steps=2)
    fes_o, asm_o = problems.build_gpu_batched(other, precision=0)
    nr_o = ikr.NewtonRaphson(asm_o, ikr.NewtonRaphsonConfig(st, ikr.LinearSolver(ikr.SolverTypeTag.gpu_PCG_Batched)))
    with pytest.raises(ikr.IkarusError, match="ARG"):
        lc.set_escalation(nr_o, ikr.FERequirements(fes_o))
    fes64, asm64 = problems.build_gpu_batched(bp, precision=0)
    nr64 = ikr.NewtonRaphson(asm64, ikr.NewtonRaphsonConfig(st, ikr.LinearSolver(ikr.SolverTypeTag.gpu_PCG_Batched)))
    with pytest.raises(ikr.IkarusError, match="ARG"):
        lc.set_escalation(nr64, ikr.FERequirements(fes))


@pytest.mark.parametrize("precision,variant", [(1, 1), (1, 2), (1, 3), (1, 4), (1, 5), (0, 1), (0, 2), (0, 3),
                                               (0, 5)])
def test_a_forced_variant_that_fits_is_the_one_launched(ikr, precision, variant):
    """Three small instances fit every kernel variant (and, in FP32, three clusters of 16 CTAs): forcing a variant
    launches that variant and no other; the planner's choice (-1) launches one of the fitting variants."""
    bp = problems.batched_cantilevers(n=3, seed=3, nx=(3, 6), nyz=(1, 2), E=(1e3, 1e4), t=(0.1, 0.3), load_steps=1)
    fes, asm = problems.build_gpu_batched(bp, precision=precision)
    st = ikr.NRSettings(tol=1e-8, maxIter=30, relative=True, linear_rtol=1e-8)
    nr = ikr.NewtonRaphson(asm, ikr.NewtonRaphsonConfig(st, ikr.LinearSolver(ikr.SolverTypeTag.gpu_PCG_Batched)))
    nr.set_batched_cg(variant=variant)
    req = ikr.FERequirements(fes)
    req.insertParameter(1.0)
    assert nr.solve(req).success
    by = nr.batched_cg_variant_launches()
    assert by[variant] > 0 and by.sum() == by[variant] == nr.batched_cg_launches()
    nr2 = ikr.NewtonRaphson(asm, ikr.NewtonRaphsonConfig(st, ikr.LinearSolver(ikr.SolverTypeTag.gpu_PCG_Batched)))
    req2 = ikr.FERequirements(fes)
    req2.insertParameter(1.0)
    assert nr2.solve(req2).success
    by2 = nr2.batched_cg_variant_launches()
    assert by2[0] == 0 and by2.sum() > 0
