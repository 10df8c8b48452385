"""GB300-native Newton-Raphson / LoadControl path for Q1 hexahedral Neo-Hookean solids.

Python front end over the C ABI of ``include/ikarus_gb300.h`` (``ikarus_gb300/_build/libikarus_gb300.so``),
with the reference's names (ikarus-project/ikarus v0.4.9): finite elements with ``calculateVector`` /
``calculateMatrix`` / ``calculateScalar``, ``FERequirements``, ``SparseFlatAssembler`` with ``DBCOption``,
``LinearSolver``, ``NewtonRaphson`` and ``LoadControl`` with observers.  All arithmetic runs in the CUDA
library on the GPU; there is no CPU path, and every call fails loudly when the library or a GPU is missing.
"""
from __future__ import annotations

import ctypes as C
import enum
import os
from dataclasses import dataclass, field

import numpy as np

from . import mesh  # noqa: F401  (re-export)

_HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(_HERE, "_build", "libikarus_gb300.so")
_lib = None


class IkarusError(RuntimeError):
    def __init__(self, code, msg):
        super().__init__(f"{_STATUS.get(code, code)}: {msg}")
        self.code = code


_STATUS = {-1: "ARG", -2: "NOT_IMPLEMENTED", -3: "INVALID_STATE", -4: "NONPOSITIVE_DETC", -5: "NOT_CONVERGED",
           -6: "CG_BREAKDOWN", -7: "CUDA", -8: "SINGULAR", -9: "NO_DEVICE", -10: "TIMEOUT"}


class DBCOption(enum.IntEnum):  # ikarus/assembler/dirichletbcenforcement.hh:8
    Raw = 0
    Reduced = 1
    Full = 2


class VectorAffordance(enum.IntEnum):  # ikarus/finiteelements/ferequirements.hh:35-89
    noAffordance = 0
    forces = 1


class MatrixAffordance(enum.IntEnum):
    noAffordance = 0
    stiffness = 1


class ScalarAffordance(enum.IntEnum):
    noAffordance = 0
    mechanicalPotentialEnergy = 1


class EAS(enum.IntEnum):  # strain measure enhanced by the EAS skill (strainenhancements/easfunctions/)
    none = 0
    GreenLagrangeStrain = 1
    DisplacementGradient = 2
    DisplacementGradientTransposed = 3


class SolverTypeTag(enum.IntEnum):  # ikarus/solver/linearsolver/linearsolver.hh:28-31 (+ device solvers)
    """The reference's 19 tags with their values (what each runs on the device: include/ikarus_gb300.h), then the
    device solvers of this library."""
    none = 0
    si_ConjugateGradient = 1
    si_LeastSquaresConjugateGradient = 2
    si_BiCGSTAB = 3
    sd_SimplicialLLT = 4
    sd_SimplicialLDLT = 5
    sd_SparseLU = 6
    sd_SparseQR = 7
    sd_CholmodSupernodalLLT = 8
    sd_UmfPackLU = 9
    sd_SuperLU = 10
    d_PartialPivLU = 11
    d_FullPivLU = 12
    d_HouseholderQR = 13
    d_ColPivHouseholderQR = 14
    d_FullPivHouseholderQR = 15
    d_CompleteOrthogonalDecomposition = 16
    d_LLT = 17
    d_LDLT = 18
    gpu_PCG_BlockJacobi = 100
    gpu_PCG_Batched = 101


DIRECT_SOLVE_RTOL = 1e-13  # IKR_DIRECT_SOLVE_RTOL: accuracy of the sparse direct tags' device solve


class Precision(enum.IntEnum):
    fp64 = 0
    fp32 = 1


class NonLinearSolverMessages(enum.IntEnum):  # ikarus/utils/broadcaster/broadcastermessages.hh:23-24
    INIT = 0
    ITERATION_STARTED = 1
    ITERATION_ENDED = 2
    RESIDUALNORM_UPDATED = 3
    CORRECTIONNORM_UPDATED = 4
    CORRECTION_UPDATED = 5
    SOLUTION_CHANGED = 6
    FINISHED_SUCESSFULLY = 7


class ControlMessages(enum.IntEnum):  # broadcastermessages.hh:18
    CONTROL_STARTED = 0
    CONTROL_ENDED = 1
    STEP_STARTED = 2
    STEP_ENDED = 3
    SOLUTION_CHANGED = 4


class _NRSettings(C.Structure):
    _fields_ = [("tol", C.c_double), ("max_iter", C.c_int32), ("min_iter", C.c_int32), ("tol_mode", C.c_int32),
                ("forcing", C.c_int32), ("linear_rtol", C.c_double), ("linear_rtol_min", C.c_double),
                ("linear_max_iter", C.c_int32), ("refinements", C.c_int32), ("max_backtracks", C.c_int32),
                ("step_graphs", C.c_int32)]


class _NRInfo(C.Structure):
    _fields_ = [("success", C.c_int32), ("residual_norm", C.c_double), ("correction_norm", C.c_double),
                ("iterations", C.c_int32), ("linear_iterations", C.c_int64)]


class _NRState(C.Structure):
    _fields_ = [("domain", C.c_void_p), ("residual_norm", C.c_double), ("correction_norm", C.c_double),
                ("iterations", C.c_int32), ("load_factor", C.c_double)]


class _ControlState(C.Structure):
    _fields_ = [("domain", C.c_void_p), ("load_step", C.c_int32), ("step_size", C.c_double),
                ("load_factor", C.c_double), ("total_iterations", C.c_int32), ("name", C.c_char_p)]


class _ControlInfo(C.Structure):
    _fields_ = [("success", C.c_int32), ("total_iterations", C.c_int32), ("n_solver_infos", C.c_int32),
                ("total_linear_iterations", C.c_int64)]


_NR_OBS = C.CFUNCTYPE(None, C.c_int32, C.POINTER(_NRState), C.c_void_p)
_LOG_SINK = C.CFUNCTYPE(None, C.c_char_p, C.c_void_p)
_POINT_FN = C.CFUNCTYPE(None, C.c_int32, C.POINTER(C.c_double), C.c_double, C.POINTER(C.c_double), C.c_void_p)


def _point_fn(fn):
    """ctypes trampoline of a load function fn(X: (n, 3) array, lambda) -> (n, 3) values."""
    def tramp(n, X, lam, out, _user):
        x = np.ctypeslib.as_array(X, shape=(n, 3))
        np.ctypeslib.as_array(out, shape=(n, 3))[:] = np.asarray(fn(x, lam), dtype=np.float64).reshape(n, 3)
    return _POINT_FN(tramp)
_CTRL_OBS = C.CFUNCTYPE(None, C.c_int32, C.POINTER(_ControlState), C.c_void_p)

# exported entry points and their ctypes signatures (kept in sync with include/ikarus_gb300.h)
_vp, _dp, _ip, _i64p, _u8p = C.c_void_p, C.POINTER(C.c_double), C.POINTER(C.c_int32), C.POINTER(C.c_int64), \
    C.POINTER(C.c_uint8)
_I, _D, _L = C.c_int32, C.c_double, C.c_int64
_fp = C.POINTER(C.c_float)
SIGNATURES = {
    "ikr_version": ([], C.c_int),
    "ikr_last_error": ([C.c_char_p, _I], C.c_int),
    "ikr_kernel_launches": ([], C.c_int64),
    "ikr_fes_create": ([C.POINTER(_vp), _I, _dp, _I, _ip, _D, _D, _I, _I], C.c_int),
    "ikr_fes_add_neumann": ([_vp, _I, _ip, _ip, _dp], C.c_int),
    "ikr_fes_destroy": ([_vp], C.c_int),
    "ikr_fes_clear_neumann": ([_vp], C.c_int),
    "ikr_fes_add_neumann_function": ([_vp, _I, _ip, _ip, _POINT_FN, _vp], C.c_int),
    "ikr_fes_add_volume_load": ([_vp, _POINT_FN, _vp], C.c_int),
    "ikr_fes_clear_volume_loads": ([_vp], C.c_int),
    "ikr_fes_set_element_materials": ([_vp, _dp, _dp], C.c_int),
    "ikr_fes_set_instances": ([_vp, _I, _ip], C.c_int),
    "ikr_newton_instance_info": ([_vp, _ip, _dp, _ip], C.c_int),
    "ikr_newton_exclude_instances": ([_vp, _I, C.POINTER(C.c_uint8)], C.c_int),
    "ikr_newton_instance_linear_iterations": ([_vp, _i64p], C.c_int),
    "ikr_newton_set_batched_cg": ([_vp, _I, _I], C.c_int),
    "ikr_newton_batched_cg_launches": ([_vp, _i64p], C.c_int),
    "ikr_newton_batched_cg_variant_launches": ([_vp, _i64p], C.c_int),
    "ikr_batched_plan_preview": ([_I, _ip, _ip, _I, _I, _ip, _I, _ip, _ip], C.c_int),
    "ikr_newton_set_batched_take_out": ([_vp, _I], C.c_int),
    "ikr_load_control_set_escalation": ([_vp, _vp, _vp], C.c_int),
    "ikr_load_control_escalated": ([_vp, _I, _u8p], C.c_int),
    "ikr_load_control_set_escalation_concurrent": ([_vp, _I], C.c_int),
    "ikr_load_control_instance_status": ([_vp, _I, _ip], C.c_int),
    "ikr_fes_num_colours": ([_vp, _ip], C.c_int),
    "ikr_fes_kernel_info": ([_vp, _ip, _ip, _ip], C.c_int),
    "ikr_fes_set_material": ([_vp, _I], C.c_int),
    "ikr_fes_set_hyperelastic": ([_vp, _vp], C.c_int),
    "ikr_assembler_set_dirichlet_values": ([_vp, _dp], C.c_int),
    "ikr_fes_get_alpha": ([_vp, _dp], C.c_int),
    "ikr_fes_set_alpha": ([_vp, _dp], C.c_int),
    "ikr_fe_calculate_vector": ([_vp, _vp, _I, _I, _I, _dp], C.c_int),
    "ikr_fe_calculate_matrix": ([_vp, _vp, _I, _I, _I, _dp], C.c_int),
    "ikr_fe_calculate_scalar": ([_vp, _vp, _I, _I, _I, _dp], C.c_int),
    "ikr_fe_update_state": ([_vp, _vp, _dp, _I], C.c_int),
    "ikr_fe_calculate_at": ([_vp, _vp, _I, _I, _I, _dp, _I, _dp], C.c_int),
    "ikr_req_create": ([C.POINTER(_vp), _vp], C.c_int),
    "ikr_req_destroy": ([_vp], C.c_int),
    "ikr_req_insert_global_solution": ([_vp, _dp], C.c_int),
    "ikr_req_global_solution": ([_vp, _dp], C.c_int),
    "ikr_req_insert_parameter": ([_vp, _D], C.c_int),
    "ikr_req_parameter": ([_vp, _dp], C.c_int),
    "ikr_req_solution_device": ([_vp, C.POINTER(_dp)], C.c_int),
    "ikr_req_copy": ([_vp, _vp], C.c_int),
    "ikr_assembler_create": ([C.POINTER(_vp), _vp, _u8p, _I], C.c_int),
    "ikr_assembler_destroy": ([_vp], C.c_int),
    "ikr_assembler_add_point_loads": ([_vp, _I, _ip, _dp], C.c_int),
    "ikr_assembler_bind": ([_vp, _vp, _I], C.c_int),
    "ikr_assembler_add_matrix_entries": ([_vp, _I, _ip, _ip, _dp], C.c_int),
    "ikr_assembler_set_dirichlet_function": ([_vp, _POINT_FN, _POINT_FN, _vp], C.c_int),
    "ikr_assembler_size": ([_vp, _ip], C.c_int),
    "ikr_assembler_reduced_size": ([_vp, _ip], C.c_int),
    "ikr_assembler_constraints_below": ([_vp, _ip], C.c_int),
    "ikr_assembler_vector": ([_vp, _vp, _I, _I, _dp], C.c_int),
    "ikr_assembler_matrix": ([_vp, _vp, _I, _I], C.c_int),
    "ikr_assembler_matrix_nnz": ([_vp, _I, _i64p], C.c_int),
    "ikr_assembler_export_csc": ([_vp, _I, _i64p, _ip, _dp], C.c_int),
    "ikr_assembler_block_pattern": ([_vp, _ip, _i64p, _ip, _ip], C.c_int),
    "ikr_assembler_vector_norm": ([_vp, _dp], C.c_int),
    "ikr_linear_solver_create": ([C.POINTER(_vp), _I], C.c_int),
    "ikr_linear_solver_destroy": ([_vp], C.c_int),
    "ikr_linear_solver_set_tolerance": ([_vp, _D, _I], C.c_int),
    "ikr_linear_solver_analyze_pattern": ([_vp, _vp], C.c_int),
    "ikr_assembler_scalar": ([_vp, _vp, _I, _dp], C.c_int),
    "ikr_nonlinear_operator_create": ([C.POINTER(_vp), _vp, _I, _I, _I, _I], C.c_int),
    "ikr_nonlinear_operator_destroy": ([_vp], C.c_int),
    "ikr_nonlinear_operator_evaluate": ([_vp, _I, _vp, _dp, _ip], C.c_int),
    "ikr_newton_residual": ([_vp, _vp, _dp], C.c_int),
    "ikr_newton_jacobian": ([_vp, _vp], C.c_int),
    "ikr_newton_update": ([_vp, _vp, _dp], C.c_int),
    "ikr_newton_subscribe_logger": ([_vp, _LOG_SINK, _vp], C.c_int),
    "ikr_newton_graph_iterations": ([_vp, _i64p], C.c_int),
    "ikr_load_control_subscribe_logger": ([_vp, _LOG_SINK, _vp], C.c_int),
    "ikr_path_following_subscribe_logger": ([_vp, _LOG_SINK, _vp], C.c_int),
    "ikr_linear_solver_set_fp64_outer": ([_vp, _I, _D, _I, _I], C.c_int),
    "ikr_linear_solver_outer_info": ([_vp, _ip, _ip], C.c_int),
    "ikr_linear_solver_set_wait_test": ([_vp, _I, _I], C.c_int),
    "ikr_linear_solver_factorize": ([_vp, _vp], C.c_int),
    "ikr_linear_solver_solve": ([_vp, _vp, _dp, _dp], C.c_int),
    "ikr_linear_solver_last_info": ([_vp, _ip, _dp], C.c_int),
    "ikr_linear_solver_profile": ([_vp, _I], C.c_int),
    "ikr_linear_solver_profile_read": ([_vp, _dp, _i64p], C.c_int),
    "ikr_linear_solver_set_launch": ([_vp, _I, _I], C.c_int),
    "ikr_linear_solver_set_kernel": ([_vp, _I, _D], C.c_int),
    "ikr_cg_kind_ranges": ([_ip], C.c_int),
    "ikr_linear_solver_kernel_info": ([_vp, _ip, _dp, _dp], C.c_int),
    "ikr_fes_stream": ([_vp, C.POINTER(_vp)], C.c_int),
    "ikr_linear_solver_solve_noalloc": ([_vp, _vp, _vp, _D, _I, _ip], C.c_int),
    "ikr_nr_settings_default": ([C.POINTER(_NRSettings)], C.c_int),
    "ikr_newton_create": ([C.POINTER(_vp), _vp, _vp, C.POINTER(_NRSettings)], C.c_int),
    "ikr_newton_destroy": ([_vp], C.c_int),
    "ikr_newton_subscribe": ([_vp, _NR_OBS, _vp], C.c_int),
    "ikr_newton_subscribe_fe_state": ([_vp, _I], C.c_int),
    "ikr_newton_solve": ([_vp, _vp, _D, C.POINTER(_NRInfo)], C.c_int),
    "ikr_load_control_create": ([C.POINTER(_vp), _vp, _I, _D, _D], C.c_int),
    "ikr_load_control_destroy": ([_vp], C.c_int),
    "ikr_load_control_subscribe": ([_vp, _CTRL_OBS, _vp], C.c_int),
    "ikr_load_control_run": ([_vp, _vp, C.POINTER(_ControlInfo), C.POINTER(_NRInfo), _I], C.c_int),
    "ikr_load_control_set_predictor": ([_vp, _I, _vp, _dp, _I], C.c_int),
    "ikr_linear_solver_set_multi_rhs": ([_vp, _I], C.c_int),
    "ikr_linear_solver_set_coarse_space": ([_vp, _I], C.c_int),
    "ikr_linear_solver_coarse_info": ([_vp, _ip], C.c_int),
    "ikr_linear_solver_set_coarse_refresh": ([_vp, _I], C.c_int),
    "ikr_assembler_set_tangent_kernel": ([_vp, _I], C.c_int),
    "ikr_assembler_tangent_kernel": ([_vp, _ip], C.c_int),
    "ikr_linear_solver_solve2": ([_vp, _vp, _dp, _dp, _dp, _dp], C.c_int),
    "ikr_path_following_create": ([C.POINTER(_vp), _vp, _I, _D, _I, _I, _ip], C.c_int),
    "ikr_path_following_destroy": ([_vp], C.c_int),
    "ikr_path_following_set_adaptive_step_sizing": ([_vp, _I, _I], C.c_int),
    "ikr_path_following_subscribe": ([_vp, _CTRL_OBS, _vp], C.c_int),
    "ikr_path_following_run": ([_vp, _vp, C.POINTER(_ControlInfo), C.POINTER(_NRInfo), _I], C.c_int),
    "ikr_path_following_subsidiary_args": ([_vp, _dp], C.c_int),
    "ikr_path_following_increment": ([_vp, _dp], C.c_int),
    "ikr_path_following_set_warm_start": ([_vp, _I], C.c_int),
    "ikr_path_following_stats": ([_vp, _dp], C.c_int),
    "ikr_load_control_predictor_stats": ([_vp, _ip, _ip], C.c_int),
    "ikr_load_control_predictor_history": ([_vp, _I, _dp, _ip], C.c_int),
    "ikr_load_control_set_predictor_gate": ([_vp, _I], C.c_int),
    "ikr_predictor_create": ([C.POINTER(_vp), _vp, _I, _I, _I, _I, _L, C.c_uint64], C.c_int),
    "ikr_predictor_destroy": ([_vp], C.c_int),
    "ikr_predictor_num_snapshots": ([_vp, _i64p], C.c_int),
    "ikr_predictor_fit": ([_vp, _I, _I, C.c_float, C.POINTER(C.c_float), _dp], C.c_int),
    "ikr_mlp_create": ([C.POINTER(_vp), _I, _I, _I, _I, C.c_uint64], C.c_int),
    "ikr_mlp_destroy": ([_vp], C.c_int),
    "ikr_mlp_num_params": ([_vp, _i64p], C.c_int),
    "ikr_mlp_get_params": ([_vp, _fp], C.c_int),
    "ikr_mlp_set_params": ([_vp, _fp], C.c_int),
    "ikr_mlp_forward": ([_vp, _I, _fp, _fp], C.c_int),
    "ikr_mlp_loss_grad": ([_vp, _I, _fp, _fp, _fp, _fp], C.c_int),
    "ikr_mlp_train": ([_vp, _I, _fp, _fp, _I, _I, C.c_float, C.c_uint64, _fp], C.c_int),
}


def lib():
    """The loaded CUDA library; raises if it was not built (there is no fallback)."""
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            raise RuntimeError(f"CUDA library missing: {LIB_PATH} (run __graft_entry__.build())")
        L = C.CDLL(LIB_PATH)
        for name, (args, res) in SIGNATURES.items():
            fn = getattr(L, name)
            fn.argtypes = args
            fn.restype = res
        _lib = L
    return _lib


def _err(code, what=""):
    if code != 0:
        buf = C.create_string_buffer(512)
        lib().ikr_last_error(buf, 512)
        raise IkarusError(code, f"{what}: {buf.value.decode(errors='replace')}")


def _ptr(a, t=C.c_double):
    return a.ctypes.data_as(C.POINTER(t))


def batched_plan_preview(rows, widths, fp32=True, variant=-1, caps=(456, 304, 304, 304, 0, 304), cluster_cap=7):
    """The batched CG's planner on given co-resident capacities (no device needed): (variant, CTAs per instance)."""
    r = np.ascontiguousarray(rows, dtype=np.int32)
    w = np.ascontiguousarray(widths, dtype=np.int32)
    cp = np.ascontiguousarray(caps, dtype=np.int32)
    v = C.c_int32()
    out = np.zeros(len(r), dtype=np.int32)
    _err(lib().ikr_batched_plan_preview(len(r), _ptr(r, C.c_int32), _ptr(w, C.c_int32), int(bool(fp32)), int(variant),
                                        _ptr(cp, C.c_int32), int(cluster_cap), C.byref(v), _ptr(out, C.c_int32)))
    return v.value, out


def kernel_launches() -> int:
    return int(lib().ikr_kernel_launches())


# ---- materials --------------------------------------------------------------------------------------------
def toLamesFirstParameterAndShearModulus(emodul: float, nu: float):
    """(E, nu) -> (lambda, mu) (ikarus/finiteelements/physicshelper.hh:81-85, 123-127, 276-280)."""
    lam = float("inf") if nu == 0.5 else emodul * nu / ((1.0 + nu) * (1.0 - 2.0 * nu))
    return lam, emodul / (2.0 * (1.0 + nu))


@dataclass
class NeoHooke:
    """Compressible Neo-Hooke law on C (materials/hyperelastic/neohooke.hh:37-208)."""
    lambda_: float
    mu: float
    kind = 0

    @classmethod
    def from_E_nu(cls, E, nu):
        return cls(*toLamesFirstParameterAndShearModulus(E, nu))


@dataclass
class StVenantKirchhoff:
    """Saint Venant-Kirchhoff law S = lambda tr(E) I + 2 mu E (materials/svk.hh:63-163)."""
    lambda_: float
    mu: float
    kind = 1

    @classmethod
    def from_E_nu(cls, E, nu):
        return cls(*toLamesFirstParameterAndShearModulus(E, nu))


@dataclass
class BlatzKo:
    """Blatz-Ko law W = mu/2 (sum 1/lambda_i^2 + 2 lambda_1 lambda_2 lambda_3 - 5) on the total principal stretches,
    no volumetric part (materials/hyperelastic/deviatoric/blatzko.hh, factory.hh:34-39 makeBlatzKo(mu))."""
    mu: float
    kind = 2

    @property
    def lambda_(self):
        return 0.0


# ---- the hyperelastic framework (materials/hyperelastic/) --------------------------------------------------
HYPER_MAX_TERMS = 4


class _HyperelasticC(C.Structure):
    """ikr_hyperelastic"""
    _fields_ = [("deviatoric", C.c_int32), ("n_terms", C.c_int32), ("mu", C.c_double * HYPER_MAX_TERMS),
                ("alpha", C.c_double * HYPER_MAX_TERMS), ("p", C.c_int32 * HYPER_MAX_TERMS),
                ("q", C.c_int32 * HYPER_MAX_TERMS), ("param", C.c_double), ("volumetric", C.c_int32),
                ("reserved", C.c_int32), ("K", C.c_double), ("beta", C.c_double)]


class PrincipalStretchTags(enum.IntEnum):
    """materials/tags.hh: the stretches an Ogden function takes"""
    total = 0
    deviatoric = 1


@dataclass(frozen=True)
class VolumetricFunction:
    """VF0..VF12 (volumetric/volumetricfunctions.hh); beta for VF4, VF7, VF10."""
    index: int
    beta: float = 0.0


def VF0():
    return VolumetricFunction(0)


def VF1():
    return VolumetricFunction(1)


def VF2():
    return VolumetricFunction(2)


def VF3():
    return VolumetricFunction(3)


def VF4(beta):
    return VolumetricFunction(4, float(beta))


def VF5():
    return VolumetricFunction(5)


def VF6():
    return VolumetricFunction(6)


def VF7(beta):
    return VolumetricFunction(7, float(beta))


def VF8():
    return VolumetricFunction(8)


def VF9():
    return VolumetricFunction(9)


def VF10(beta):
    return VolumetricFunction(10, float(beta))


def VF11():
    return VolumetricFunction(11)


def VF12():
    return VolumetricFunction(12)


@dataclass
class Hyperelastic:
    """Hyperelastic<Deviatoric<DF>, Volumetric<VF>> (materials/hyperelastic/interface.hh): W(C) = W_dev(lambda_1,
    lambda_2, lambda_3) + K U(J).  ``deviatoric`` is one of the DEV_* codes below with its parameters; build it with the
    factories (makeOgden, makeMooneyRivlin, makeYeoh, makeInvariantBased, makeArrudaBoyce, makeGent, makeBlatzKo,
    makePureVolumetric; hyperelastic/factory.hh)."""
    deviatoric: int
    mu: tuple = ()
    alpha: tuple = ()
    p: tuple = ()
    q: tuple = ()
    param: float = 0.0
    K: float = 0.0
    vf: VolumetricFunction = VolumetricFunction(0)
    kind = 3
    lambda_ = 0.0

    DEV_NONE, DEV_BLATZKO, DEV_OGDEN_TOTAL, DEV_OGDEN_DEVIATORIC = 0, 1, 2, 3
    DEV_INVARIANT_BASED, DEV_ARRUDA_BOYCE, DEV_GENT = 4, 5, 6

    def _c(self):
        h = _HyperelasticC()
        h.deviatoric, h.n_terms = int(self.deviatoric), max(1, len(self.mu))
        for name in ("mu", "alpha", "p", "q"):
            vals = getattr(self, name)
            if len(vals) > HYPER_MAX_TERMS:
                raise IkarusError(-1, f"at most {HYPER_MAX_TERMS} terms")
            for i, v in enumerate(vals):
                getattr(h, name)[i] = v
        h.param, h.volumetric, h.K, h.beta = float(self.param), int(self.vf.index), float(self.K), float(self.vf.beta)
        return h

    def oracle_terms(self):
        """The plain values of the description (keyword arguments of the oracle's ``hyper``)."""
        return dict(deviatoric=int(self.deviatoric), mu=list(self.mu), alpha=list(self.alpha), p=list(self.p),
                    q=list(self.q), param=float(self.param), volumetric=int(self.vf.index), K=float(self.K),
                    beta=float(self.vf.beta))

    @property
    def mu0(self):
        return float(self.mu[0]) if self.mu else 0.0


def makeBlatzKo(mu, K=0.0, vf=None):
    """makeBlatzKo(mu) (factory.hh:34-39); K and vf add a volumetric part as Hyperelastic(dev, vol) would."""
    return Hyperelastic(Hyperelastic.DEV_BLATZKO, mu=(float(mu),), K=K, vf=vf or VF0())


def makeOgden(mu, alpha, K=0.0, vf=None, tag=PrincipalStretchTags.total):
    """makeOgden<n, tag>(mu, alpha, K, vf) (factory.hh:52-61)."""
    if len(mu) != len(alpha):
        raise IkarusError(-1, "Ogden: as many exponents as moduli")
    dev = Hyperelastic.DEV_OGDEN_TOTAL if tag == PrincipalStretchTags.total else Hyperelastic.DEV_OGDEN_DEVIATORIC
    return Hyperelastic(dev, mu=tuple(map(float, mu)), alpha=tuple(map(float, alpha)), K=K, vf=vf or VF0())


def makeInvariantBased(mu, pex, qex, K=0.0, vf=None):
    """makeInvariantBased<n>(mu, p, q, K, vf) (factory.hh:74-83): W = sum mu_i (W1 - 3)^p_i (W2 - 3)^q_i."""
    if not (len(mu) == len(pex) == len(qex)):
        raise IkarusError(-1, "InvariantBased: as many exponents as coefficients")
    return Hyperelastic(Hyperelastic.DEV_INVARIANT_BASED, mu=tuple(map(float, mu)), p=tuple(map(int, pex)),
                        q=tuple(map(int, qex)), K=K, vf=vf or VF0())


def makeMooneyRivlin(mu, K=0.0, vf=None):
    """makeMooneyRivlin(mu, K, vf) (factory.hh:96-102): p = {1, 0}, q = {0, 1}."""
    return makeInvariantBased(mu, (1, 0), (0, 1), K, vf)


def makeYeoh(mu, K=0.0, vf=None):
    """makeYeoh(mu, K, vf) (factory.hh:115-121): p = {1, 2, 3}, q = {0, 0, 0}."""
    return makeInvariantBased(mu, (1, 2, 3), (0, 0, 0), K, vf)


def makeArrudaBoyce(mu, lambdaM, K=0.0, vf=None):
    """makeArrudaBoyce({mu, lambdaM}, K, vf) (factory.hh:133-140)."""
    return Hyperelastic(Hyperelastic.DEV_ARRUDA_BOYCE, mu=(float(mu),), param=float(lambdaM), K=K, vf=vf or VF0())


def makeGent(mu, Jm, K=0.0, vf=None):
    """makeGent({mu, Jm}, K, vf) (factory.hh:152-158)."""
    return Hyperelastic(Hyperelastic.DEV_GENT, mu=(float(mu),), param=float(Jm), K=K, vf=vf or VF0())


def makePureVolumetric(vf, K):
    """makePureVolumetric(vf, K) (factory.hh:169-174): no deviatoric part."""
    return Hyperelastic(Hyperelastic.DEV_NONE, K=float(K), vf=vf)


# ---- finite elements -------------------------------------------------------------------------------------
class FiniteElements:
    """All elements of one Q1 hexahedral mesh with skills nonLinearElastic(NeoHooke) [+ eas<ES>(n)]
    [+ neumannBoundaryLoad], bound to their grid elements (the reference's ``std::vector<FE>``)."""

    def __init__(self, coords, conn, material, eas: EAS = EAS.none, n_eas: int = 0):
        self.coords = np.ascontiguousarray(coords, dtype=np.float64)
        self.conn = np.ascontiguousarray(conn, dtype=np.int32)
        self.n_nodes, self.n_elems = self.coords.shape[0], self.conn.shape[0]
        self.n_dofs = 3 * self.n_nodes
        self.n_eas = int(n_eas)
        self.material = material
        h = C.c_void_p()
        mu = material.mu0 if isinstance(material, Hyperelastic) else material.mu
        _err(lib().ikr_fes_create(C.byref(h), self.n_nodes, _ptr(self.coords), self.n_elems,
                                  _ptr(self.conn, C.c_int32), material.lambda_, mu, int(eas), self.n_eas),
             "fes_create")
        self.h = h
        self._load_cbs = []  # ctypes trampolines of function-defined loads (kept alive with the element set)
        if isinstance(material, Hyperelastic):
            self._hyper = material._c()
            _err(lib().ikr_fes_set_hyperelastic(self.h, C.byref(self._hyper)), "set_hyperelastic")
        elif getattr(material, "kind", 0):
            _err(lib().ikr_fes_set_material(self.h, int(material.kind)), "set_material")

    def __del__(self):
        if getattr(self, "h", None) and _lib is not None:
            _lib.ikr_fes_destroy(self.h)
            self.h = None

    def add_neumann(self, face_elem, face_local, traction):
        """neumannBoundaryLoad: traction per face (n_faces x 3, value at the face centre, load factor 1)."""
        fe = np.ascontiguousarray(face_elem, dtype=np.int32)
        fl = np.ascontiguousarray(face_local, dtype=np.int32)
        t = np.ascontiguousarray(np.broadcast_to(np.asarray(traction, dtype=np.float64), (len(fe), 3)))
        _err(lib().ikr_fes_add_neumann(self.h, len(fe), _ptr(fe, C.c_int32), _ptr(fl, C.c_int32), _ptr(t)),
             "add_neumann")

    def add_neumann_function(self, face_elem, face_local, fn):
        """neumannBoundaryLoad(patch, f) with f(X, lambda): fn(X (n, 3), lambda) -> tractions (n, 3) at the faces'
        quadrature points (face centres), evaluated whenever the load factor changes."""
        fe = np.ascontiguousarray(face_elem, dtype=np.int32)
        fl = np.ascontiguousarray(face_local, dtype=np.int32)
        cb = _point_fn(fn)
        self._load_cbs.append(cb)
        _err(lib().ikr_fes_add_neumann_function(self.h, len(fe), _ptr(fe, C.c_int32), _ptr(fl, C.c_int32), cb,
                                                None), "add_neumann_function")

    def add_volume_load(self, fn):
        """volumeLoad(f) (loads/volume.hh): fn(X (n, 3), lambda) -> body forces (n, 3) at the Gauss points."""
        cb = _point_fn(fn)
        self._load_cbs.append(cb)
        _err(lib().ikr_fes_add_volume_load(self.h, cb, None), "add_volume_load")

    def clear_volume_loads(self):
        _err(lib().ikr_fes_clear_volume_loads(self.h))

    def clear_neumann(self):
        _err(lib().ikr_fes_clear_neumann(self.h), "clear_neumann")

    def set_element_materials(self, lam, mu):
        """Per-element NeoHooke Lame parameters."""
        lam = np.ascontiguousarray(lam, dtype=np.float64)
        mu = np.ascontiguousarray(mu, dtype=np.float64)
        _err(lib().ikr_fes_set_element_materials(self.h, _ptr(lam), _ptr(mu)), "set_element_materials")

    def set_instances(self, node_offsets):
        """Independent problems on contiguous node ranges (batched Newton / CG with gpu_PCG_Batched)."""
        off = np.ascontiguousarray(node_offsets, dtype=np.int32)
        self.n_instances = len(off) - 1
        _err(lib().ikr_fes_set_instances(self.h, self.n_instances, _ptr(off, C.c_int32)), "set_instances")

    def kernel_info(self):
        """Elements per block of the element kernel for residual / FP64 tangent / FP32 tangent (0: not yet)."""
        a, b, c = C.c_int32(), C.c_int32(), C.c_int32()
        _err(lib().ikr_fes_kernel_info(self.h, C.byref(a), C.byref(b), C.byref(c)))
        return a.value, b.value, c.value

    def num_colours(self):
        n = C.c_int32()
        _err(lib().ikr_fes_num_colours(self.h, C.byref(n)))
        return n.value

    def stream(self) -> int:
        """Address of the cudaStream_t the library issues this element set's work on."""
        s = C.c_void_p()
        _err(lib().ikr_fes_stream(self.h, C.byref(s)))
        return int(s.value or 0)

    @property
    def alpha(self):
        a = np.zeros((self.n_elems, self.n_eas))
        if a.size:
            _err(lib().ikr_fes_get_alpha(self.h, _ptr(a)), "get_alpha")
        return a

    @alpha.setter
    def alpha(self, a):
        a = np.ascontiguousarray(a, dtype=np.float64)
        _err(lib().ikr_fes_set_alpha(self.h, _ptr(a)), "set_alpha")


class FERequirements:
    """Displacement (device-resident FP64) and load factor (ferequirements.hh:222-407)."""

    def __init__(self, fes: FiniteElements, u=None, load_factor: float = 0.0):
        self.fes = fes
        h = C.c_void_p()
        _err(lib().ikr_req_create(C.byref(h), fes.h), "req_create")
        self.h = h
        if u is not None:
            self.insertGlobalSolution(u)
        self.insertParameter(load_factor)

    def __del__(self):
        if getattr(self, "h", None) and _lib is not None:
            _lib.ikr_req_destroy(self.h)
            self.h = None

    def insertGlobalSolution(self, u):
        u = np.ascontiguousarray(u, dtype=np.float64)
        if u.size != self.fes.n_dofs:
            raise ValueError("solution size mismatch")
        _err(lib().ikr_req_insert_global_solution(self.h, _ptr(u)), "insertGlobalSolution")

    def globalSolution(self):
        u = np.zeros(self.fes.n_dofs)
        _err(lib().ikr_req_global_solution(self.h, _ptr(u)), "globalSolution")
        return u

    def insertParameter(self, lf: float):
        _err(lib().ikr_req_insert_parameter(self.h, float(lf)), "insertParameter")

    def parameter(self) -> float:
        v = C.c_double()
        _err(lib().ikr_req_parameter(self.h, C.byref(v)), "parameter")
        return v.value

    def assign(self, other: "FERequirements"):
        """Deep copy of another requirement's solution and load factor, device to device."""
        _err(lib().ikr_req_copy(self.h, other.h), "copy")


def calculateVector(fes: FiniteElements, req: FERequirements, affordance=VectorAffordance.forces, elements=None):
    """Element force vectors (n x 24) of the given element range (mixin.hh:137-140)."""
    e0, e1 = elements if elements is not None else (0, fes.n_elems)
    out = np.zeros((e1 - e0, 24))
    _err(lib().ikr_fe_calculate_vector(fes.h, req.h, int(affordance), e0, e1, _ptr(out)), "calculateVector")
    return out


def calculateMatrix(fes: FiniteElements, req: FERequirements, affordance=MatrixAffordance.stiffness, elements=None):
    """Element stiffness matrices (n x 24 x 24) of the given element range (mixin.hh:149-152)."""
    e0, e1 = elements if elements is not None else (0, fes.n_elems)
    out = np.zeros((e1 - e0, 576))
    _err(lib().ikr_fe_calculate_matrix(fes.h, req.h, int(affordance), e0, e1, _ptr(out)), "calculateMatrix")
    return out.reshape(-1, 24, 24).transpose(0, 2, 1).copy()  # stored column-major


def calculateScalar(fes: FiniteElements, req: FERequirements,
                    affordance=ScalarAffordance.mechanicalPotentialEnergy, elements=None):
    e0, e1 = elements if elements is not None else (0, fes.n_elems)
    out = np.zeros(e1 - e0)
    _err(lib().ikr_fe_calculate_scalar(fes.h, req.h, int(affordance), e0, e1, _ptr(out)), "calculateScalar")
    return out


class ResultTypes(enum.IntEnum):  # feresulttypes.hh:125-128 (the stresses of the nonlinear-elastic element)
    PK2Stress = 0
    kirchhoffStress = 1
    cauchyStress = 2


def calculateAt(fes: FiniteElements, req: FERequirements, result_type: ResultTypes, local=(0.5, 0.5, 0.5),
                elements=None):
    """Stress at local points of the reference cube (nonlinearelastic.hh:237-271): one point for all elements or
    one per element (n x 3); returns n x 6 Voigt values [11, 22, 33, 23, 13, 12]."""
    e0, e1 = elements if elements is not None else (0, fes.n_elems)
    loc = np.ascontiguousarray(local, dtype=np.float64)
    per = loc.ndim == 2
    if per and loc.shape != (e1 - e0, 3):
        raise ValueError("one local point per element expected")
    out = np.zeros((e1 - e0, 6))
    _err(lib().ikr_fe_calculate_at(fes.h, req.h, int(result_type), e0, e1, _ptr(loc), int(per), _ptr(out)),
         "calculateAt")
    return out


def updateState(fes: FiniteElements, req: FERequirements, correction):
    c = np.ascontiguousarray(correction, dtype=np.float64)
    _err(lib().ikr_fe_update_state(fes.h, req.h, _ptr(c), c.size), "updateState")


# ---- assembler -------------------------------------------------------------------------------------------
class SparseFlatAssembler:
    """SparseFlatAssembler (simpleassemblers.hh:108-177) with Dirichlet flags and manipulator point loads."""

    def __init__(self, fes: FiniteElements, fixed_dofs, precision: Precision = Precision.fp64):
        self.fes = fes
        fixed = np.ascontiguousarray(fixed_dofs, dtype=np.uint8)
        if fixed.size != fes.n_dofs:
            raise ValueError("Dirichlet flag size mismatch")
        self.fixed = fixed
        self.precision = Precision(precision)
        h = C.c_void_p()
        _err(lib().ikr_assembler_create(C.byref(h), fes.h, _ptr(fixed, C.c_uint8), int(precision)), "assembler")
        self.h = h
        self._req = None
        self._dbc = DBCOption.Full

    def __del__(self):
        if getattr(self, "h", None) and _lib is not None:
            _lib.ikr_assembler_destroy(self.h)
            self.h = None

    def bind(self, req: FERequirements, dbc: DBCOption = DBCOption.Full):
        _err(lib().ikr_assembler_bind(self.h, req.h, int(dbc)), "bind")
        self._req, self._dbc = req, DBCOption(dbc)

    def dBCOption(self):
        return self._dbc

    def add_point_loads(self, dofs, values):
        """AssemblerManipulator vector hook: vec[dof] += load_factor * value after the Dirichlet treatment."""
        d = np.ascontiguousarray(dofs, dtype=np.int32)
        v = np.ascontiguousarray(values, dtype=np.float64)
        _err(lib().ikr_assembler_add_point_loads(self.h, len(d), _ptr(d, C.c_int32), _ptr(v)), "point loads")

    def set_dirichlet_function(self, value, derivative):
        """storeInhomogeneousBoundaryCondition(f): value(X (n, 3), lambda) -> prescribed displacements at every node
        (nonzero entries are imposed), derivative(X, lambda) -> their lambda-derivative (used at lambda = 1)."""
        cv, cd = _point_fn(value), _point_fn(derivative)
        self._dirichlet_cbs = (cv, cd)
        _err(lib().ikr_assembler_set_dirichlet_function(self.h, cv, cd, None), "set_dirichlet_function")

    def add_matrix_entries(self, rows, cols, values):
        """AssemblerManipulator matrix hook: K(row, col) += value after every assembly (springs)."""
        r = np.ascontiguousarray(rows, dtype=np.int32)
        c = np.ascontiguousarray(cols, dtype=np.int32)
        v = np.ascontiguousarray(values, dtype=np.float64)
        _err(lib().ikr_assembler_add_matrix_entries(self.h, len(r), _ptr(r, C.c_int32), _ptr(c, C.c_int32), _ptr(v)),
             "add_matrix_entries")

    def size(self):
        return self.fes.n_dofs

    def reducedSize(self):
        n = C.c_int32()
        _err(lib().ikr_assembler_reduced_size(self.h, C.byref(n)))
        return n.value

    def constraintsBelow(self):
        out = np.zeros(self.size(), dtype=np.int32)
        _err(lib().ikr_assembler_constraints_below(self.h, _ptr(out, C.c_int32)))
        return out

    def isConstrained(self, i):
        return bool(self.fixed[i])

    def createFullVector(self, reduced):
        full = np.zeros(self.size())
        full[self.fixed == 0] = reduced
        return full

    def createReducedVector(self, full):
        return np.asarray(full)[self.fixed == 0].copy()

    def _args(self, req, dbc):
        req = req if req is not None else self._req
        if req is None:
            raise IkarusError(-3, "assembler not bound")
        return req, DBCOption(self._dbc if dbc is None else dbc)

    def set_tangent_kernel(self, path=0):
        """FP32 displacement-based tangent: 1 coloured element kernel, 2 row kernel, 3 element blocks + gather, 0 timed
        choice."""
        _err(lib().ikr_assembler_set_tangent_kernel(self.h, int(path)))

    def tangent_kernel(self):
        """The FP32 tangent kernel in use (0 = not chosen yet, 1 coloured, 2 rows)."""
        v = C.c_int32()
        _err(lib().ikr_assembler_tangent_kernel(self.h, C.byref(v)))
        return v.value

    def set_dirichlet_values(self, rate):
        """Inhomogeneous Dirichlet values lambda * rate on constrained dofs (storeInhomogeneousBoundaryCondition for
        values linear in the load factor); None removes them."""
        if rate is None:
            _err(lib().ikr_assembler_set_dirichlet_values(self.h, None), "set_dirichlet_values")
            return
        r = np.ascontiguousarray(rate, dtype=np.float64)
        if r.size != self.size():
            raise ValueError("Dirichlet value size mismatch")
        _err(lib().ikr_assembler_set_dirichlet_values(self.h, _ptr(r)), "set_dirichlet_values")

    def vector(self, req=None, affordance=VectorAffordance.forces, dbc=None, export=True):
        """Assembles on the device; returns the host copy unless export=False."""
        req, dbc = self._args(req, dbc)
        if not export:
            _err(lib().ikr_assembler_vector(self.h, req.h, int(affordance), int(dbc), None), "vector")
            return None
        n = self.reducedSize() if dbc == DBCOption.Reduced else self.size()
        out = np.zeros(n)
        _err(lib().ikr_assembler_vector(self.h, req.h, int(affordance), int(dbc), _ptr(out)), "vector")
        return out

    def matrix(self, req=None, affordance=MatrixAffordance.stiffness, dbc=None, export=True):
        """Assembles on the device; returns the scalar CSC (scipy) unless export=False."""
        req, dbc = self._args(req, dbc)
        _err(lib().ikr_assembler_matrix(self.h, req.h, int(affordance), int(dbc)), "matrix")
        return self.export_csc(dbc) if export else None

    def export_csc(self, dbc=None):
        import scipy.sparse as sp
        dbc = DBCOption(self._dbc if dbc is None else dbc)
        nnz = C.c_int64()
        _err(lib().ikr_assembler_matrix_nnz(self.h, int(dbc), C.byref(nnz)), "nnz")
        n = self.reducedSize() if dbc == DBCOption.Reduced else self.size()
        cp = np.zeros(n + 1, dtype=np.int64)
        ri = np.zeros(nnz.value, dtype=np.int32)
        v = np.zeros(nnz.value)
        _err(lib().ikr_assembler_export_csc(self.h, int(dbc), _ptr(cp, C.c_int64), _ptr(ri, C.c_int32), _ptr(v)),
             "export")
        return sp.csc_matrix((v, ri, cp), shape=(n, n))

    def pattern_csc(self, dbc=DBCOption.Full):
        nnz = C.c_int64()
        _err(lib().ikr_assembler_matrix_nnz(self.h, int(dbc), C.byref(nnz)), "nnz")
        n = self.reducedSize() if dbc == DBCOption.Reduced else self.size()
        cp = np.zeros(n + 1, dtype=np.int64)
        ri = np.zeros(nnz.value, dtype=np.int32)
        _err(lib().ikr_assembler_export_csc(self.h, int(dbc), _ptr(cp, C.c_int64), _ptr(ri, C.c_int32), None),
             "pattern")
        return cp, ri

    def block_pattern(self):
        nr, nb = C.c_int32(), C.c_int64()
        _err(lib().ikr_assembler_block_pattern(self.h, C.byref(nr), C.byref(nb), None, None))
        rp = np.zeros(nr.value + 1, dtype=np.int32)
        col = np.zeros(nb.value, dtype=np.int32)
        _err(lib().ikr_assembler_block_pattern(self.h, None, None, _ptr(rp, C.c_int32), _ptr(col, C.c_int32)))
        return rp, col

    def vector_norm(self):
        v = C.c_double()
        _err(lib().ikr_assembler_vector_norm(self.h, C.byref(v)))
        return v.value

    def scalar(self, req=None, affordance=ScalarAffordance.mechanicalPotentialEnergy):
        """scalar(req, affordance): the sum of the element energies in element order (simpleassemblers.inl)."""
        req, _ = self._args(req, None)
        v = C.c_double()
        _err(lib().ikr_assembler_scalar(self.h, req.h, int(affordance), C.byref(v)), "scalar")
        return v.value


# ---- NonLinearOperator ------------------------------------------------------------------------------------
@dataclass(frozen=True)
class AffordanceCollection:  # ferequirements.hh:35-89, 205-208
    scalarAffordance: ScalarAffordance = ScalarAffordance.noAffordance
    vectorAffordance: VectorAffordance = VectorAffordance.forces
    matrixAffordance: MatrixAffordance = MatrixAffordance.stiffness

    @property
    def hasScalarAffordance(self):
        return self.scalarAffordance != ScalarAffordance.noAffordance


class AffordanceCollections:
    elastoStatics = AffordanceCollection(ScalarAffordance.mechanicalPotentialEnergy, VectorAffordance.forces,
                                         MatrixAffordance.stiffness)


class DifferentiableFunction:
    """One derivative order of the non-linear operator: f(req) returns the energy (float), the force vector
    (numpy) or the tangent (scipy CSC exported from the assembler's device storage)."""

    def __init__(self, op, order):
        self._op, self.order = op, order

    def __call__(self, req):
        a = self._op.assembler
        kind = C.c_int32()
        if self._op.kind_of(self.order) == 1:
            n = a.reducedSize() if self._op.dbcOption == DBCOption.Reduced else a.size()
            out = np.zeros(n)
            _err(lib().ikr_nonlinear_operator_evaluate(self._op.h, self.order, req.h, _ptr(out), C.byref(kind)), "op")
            return out
        v = C.c_double()
        _err(lib().ikr_nonlinear_operator_evaluate(self._op.h, self.order, req.h, C.byref(v), C.byref(kind)), "op")
        return v.value if kind.value == 0 else a.export_csc(self._op.dbcOption)

    def derivative(self):
        return DifferentiableFunction(self._op, self.order + 1)


def derivative(f: DifferentiableFunction) -> DifferentiableFunction:
    """derivative(f) of the reference's DifferentiableFunction (differentiablefunction.hh:60-87)."""
    return f.derivative()


class _NonLinearOperator:
    def __init__(self, assembler, affordances: AffordanceCollection, dbcOption: DBCOption):
        h = C.c_void_p()
        _err(lib().ikr_nonlinear_operator_create(C.byref(h), assembler.h, int(affordances.scalarAffordance),
                                                 int(affordances.vectorAffordance),
                                                 int(affordances.matrixAffordance), int(dbcOption)), "op")
        self.h, self.assembler, self.affordances, self.dbcOption = h, assembler, affordances, DBCOption(dbcOption)

    def __del__(self):
        if getattr(self, "h", None) and _lib is not None:
            _lib.ikr_nonlinear_operator_destroy(self.h)
            self.h = None

    def kind_of(self, order):
        return order if self.affordances.hasScalarAffordance else order + 1


class DifferentiableFunctionFactory:  # utils/differentiablefunctionfactory.hh:22-65
    @staticmethod
    def op(assembler, affordances: AffordanceCollection = None, dbcOption: DBCOption = DBCOption.Full):
        """The non-linear operator over the assembler: energy -> forces -> stiffness with a scalar affordance in the
        collection, forces -> stiffness without.  Returns f; derivative(f) is the next order."""
        if affordances is None:
            affordances = AffordanceCollection()
        return DifferentiableFunction(_NonLinearOperator(assembler, affordances, dbcOption), 0)


# ---- listeners --------------------------------------------------------------------------------------------
class _Logger:
    def __init__(self, sink=None):
        """sink(line) receives every line; None prints through the library ("[info] <line>" on stdout)."""
        self.lines = []
        self._sink = sink

        def tramp(line, _user):
            text = line.decode()
            self.lines.append(text)
            if self._sink is not None:
                self._sink(text)
        self._cb = _LOG_SINK(tramp) if sink is not None else _LOG_SINK()
        self._subscribed = []

    def _cb_for(self):
        return self._cb


class NonLinearSolverLogger(_Logger):
    """NonLinearSolverLogger (utils/listener/nonlinearsolverlogger.hh:22-95)."""

    def subscribeTo(self, nr: "NewtonRaphson"):
        _err(lib().ikr_newton_subscribe_logger(nr.h, self._cb, None), "logger")
        self._subscribed.append(nr)
        return self


class ControlLogger(_Logger):
    """ControlLogger (utils/listener/controllogger.hh:22-66)."""

    def subscribeTo(self, control):
        fn = lib().ikr_path_following_subscribe_logger if isinstance(control, PathFollowing) else \
            lib().ikr_load_control_subscribe_logger
        _err(fn(control.h, self._cb, None), "logger")
        self._subscribed.append(control)
        return self


# ---- solvers ---------------------------------------------------------------------------------------------
class LinearSolver:
    """LinearSolver facade (linearsolver.hh:49-233) over the device CG solvers."""

    def __init__(self, tag: SolverTypeTag = SolverTypeTag.gpu_PCG_BlockJacobi, rtol=None, max_iter=100000):
        h = C.c_void_p()
        _err(lib().ikr_linear_solver_create(C.byref(h), int(tag)), "linear solver")
        self.h = h
        self.tag = tag
        if rtol is None:  # the sparse direct tags default to a direct solver's accuracy
            rtol = DIRECT_SOLVE_RTOL if SolverTypeTag.sd_SimplicialLLT <= tag <= SolverTypeTag.sd_UmfPackLU else 1e-10
        self.setTolerance(rtol, max_iter)

    def __del__(self):
        if getattr(self, "h", None) and _lib is not None:
            _lib.ikr_linear_solver_destroy(self.h)
            self.h = None

    def setTolerance(self, rtol, max_iter=100000):
        _err(lib().ikr_linear_solver_set_tolerance(self.h, rtol, max_iter))
        self.rtol, self.max_iter = rtol, max_iter

    def analyzePattern(self, assembler: SparseFlatAssembler):
        _err(lib().ikr_linear_solver_analyze_pattern(self.h, assembler.h), "analyzePattern")

    def factorize(self, assembler: SparseFlatAssembler):
        _err(lib().ikr_linear_solver_factorize(self.h, assembler.h), "factorize")

    def compute(self, assembler: SparseFlatAssembler):
        self.analyzePattern(assembler)
        self.factorize(assembler)

    def solve(self, assembler: SparseFlatAssembler, b):
        """x = K^-1 b; b of shape (n,) or (n, 2) (two columns, as the path-following Newton solves them)."""
        b = np.asarray(b, dtype=np.float64)
        if b.ndim == 2:
            if b.shape[1] != 2:
                raise ValueError("two right-hand-side columns are supported")
            b0, b1 = np.ascontiguousarray(b[:, 0]), np.ascontiguousarray(b[:, 1])
            x0, x1 = np.zeros_like(b0), np.zeros_like(b1)
            _err(lib().ikr_linear_solver_solve2(self.h, assembler.h, _ptr(x0), _ptr(x1), _ptr(b0), _ptr(b1)),
                 "solve")
            return np.stack([x0, x1], axis=1)
        b = np.ascontiguousarray(b)
        x = np.zeros_like(b)
        _err(lib().ikr_linear_solver_solve(self.h, assembler.h, _ptr(x), _ptr(b)), "solve")
        return x

    def last_info(self):
        it, rel = C.c_int32(), C.c_double()
        _err(lib().ikr_linear_solver_last_info(self.h, C.byref(it), C.byref(rel)))
        return it.value, rel.value

    def profile(self, on=True):
        """Bracket every CG SpMV with device events (inside the CUDA graphs); resets the counters."""
        _err(lib().ikr_linear_solver_profile(self.h, int(on)))

    def set_launch(self, use_graphs=True, chunk_len=16):
        """CG iterations per host poll, issued as CUDA graphs or kernel by kernel."""
        _err(lib().ikr_linear_solver_set_launch(self.h, int(use_graphs), int(chunk_len)))

    @staticmethod
    def kind_ranges():
        """{"staged", "persistent", "coarse_fused", "count"}: the first CG kind of each family and the number of kinds."""
        out = (C.c_int32 * 4)()
        _err(lib().ikr_cg_kind_ranges(out))
        return dict(zip(("staged", "persistent", "coarse_fused", "count"), list(out)))

    def set_kernel(self, spmv_kind=-1, l2_keep_fraction=-1.0):
        """CG kernel (0 direct-load SpMV, then the staged, persistent and fused-coarse kinds of ``kind_ranges``; -1
        autotune) and L2 keep fraction (-1 autotune)."""
        _err(lib().ikr_linear_solver_set_kernel(self.h, int(spmv_kind), float(l2_keep_fraction)))

    def set_multi_rhs(self, on=True):
        """Two right-hand sides with one tangent (path following): one persistent launch streaming the matrix once
        per iteration for both (default), or one solve after the other."""
        _err(lib().ikr_linear_solver_set_multi_rhs(self.h, int(bool(on))))

    def set_fp64_outer(self, restart=20, inner_rtol=1e-2, inner_max_iter=2000, outer_max_iter=2000):
        """FP64 outer solve of an FP32 tangent (restart 0 switches it off): flexible GMRES(restart) on the FP64
        tangent, right-preconditioned by the FP32 block-Jacobi CG (to inner_rtol, at most inner_max_iter iterations
        per application) on the FP32 rounding of the same tangent."""
        _err(lib().ikr_linear_solver_set_fp64_outer(self.h, int(restart), float(inner_rtol), int(inner_max_iter),
                                                    int(outer_max_iter)))

    def set_wait_test(self, barrier_polls=0, withhold_first_arrival=False):
        """Test hook of the bounded device waits: grid-barrier poll limit of the persistent CG (0 = default) and a
        one-launch switch that withholds CTA 0's first barrier arrival (the solve then reports the timeout)."""
        _err(lib().ikr_linear_solver_set_wait_test(self.h, int(barrier_polls), int(bool(withhold_first_arrival))))

    def outer_info(self):
        """(Arnoldi steps, restart cycles) of the last FP64 outer solve."""
        o, c = C.c_int32(), C.c_int32()
        _err(lib().ikr_linear_solver_outer_info(self.h, C.byref(o), C.byref(c)))
        return o.value, c.value

    def set_coarse_space(self, n_slabs):
        """Coarse correction of the block-Jacobi CG (0 = off, the default): n_slabs in [1, 128] slabs of equal node
        count along the mesh's longest extent, six rigid-body modes each, A_c = P^T K P rebuilt at every
        factorize (an additive two-level preconditioner; two-kernel CG forms, or with at most 64 slabs the persistent
        kernel with the correction fused in, which the tuner prefers)."""
        _err(lib().ikr_linear_solver_set_coarse_space(self.h, int(n_slabs)))

    def set_coarse_refresh(self, every):
        """Rebuild A_c at every ``every``-th factorize only (1, the default: each time); in between the coarse
        operator of an earlier tangent stays (still SPD: same solution, possibly more CG iterations)."""
        _err(lib().ikr_linear_solver_set_coarse_refresh(self.h, int(every)))

    def coarse_info(self):
        """{"slabs", "coarse_dofs", "dropped_modes", "colours"} of the coarse correction in use (zeros when off)."""
        out = (C.c_int32 * 4)()
        _err(lib().ikr_linear_solver_coarse_info(self.h, out))
        return dict(zip(("slabs", "coarse_dofs", "dropped_modes", "colours"), list(out)))

    def kernel_info(self):
        """(spmv kind, L2 keep fraction, tuned SpMV microseconds per launch)."""
        k, f, us = C.c_int32(), C.c_double(), C.c_double()
        _err(lib().ikr_linear_solver_kernel_info(self.h, C.byref(k), C.byref(f), C.byref(us)))
        return k.value, f.value, us.value

    def profile_read(self):
        """(summed SpMV device time in ms, SpMV launches) since profiling was switched on."""
        ms, n = C.c_double(), C.c_int64()
        _err(lib().ikr_linear_solver_profile_read(self.h, C.byref(ms), C.byref(n)))
        return ms.value, n.value


@dataclass
class NRSettings:
    """NRSettings (newtonraphson.hh:27-32) plus the inexact-Newton controls of this library."""
    tol: float = 1e-8
    maxIter: int = 20
    minIter: int = 0
    relative: bool = False        # ||R|| <= tol * ||R0|| instead of the reference's absolute test
    eisenstat_walker: bool = False
    linear_rtol: float = 1e-10
    linear_rtol_min: float = 1e-12
    linear_max_iter: int = 100000
    refinements: int = 0
    backtracks: int = 0           # halve a correction that inverts an element (the reference aborts)
    step_graphs: bool = True      # each Newton iteration as one CUDA graph launch where the configuration allows it

    def _c(self):
        return _NRSettings(self.tol, self.maxIter, self.minIter, int(self.relative), int(self.eisenstat_walker),
                           self.linear_rtol, self.linear_rtol_min, self.linear_max_iter, self.refinements,
                           self.backtracks, int(self.step_graphs))


@dataclass
class NonLinearSolverInformation:  # solverinfos.hh:20-32
    success: bool = False
    residualNorm: float = float("inf")
    correctionNorm: float = float("inf")
    iterations: int = -1
    linearIterations: int = 0

    def __bool__(self):
        return self.success

    @classmethod
    def _from(cls, c: _NRInfo):
        return cls(bool(c.success), c.residual_norm, c.correction_norm, c.iterations, c.linear_iterations)


@dataclass
class NewtonRaphsonConfig:  # newtonraphson.hh:38-70
    parameters: NRSettings = field(default_factory=NRSettings)
    linearSolver: LinearSolver = None


class NewtonRaphson:
    """NewtonRaphson (newtonraphson.hh:193-257), a broadcaster of NonLinearSolverMessages."""

    def __init__(self, assembler: SparseFlatAssembler, config: NewtonRaphsonConfig):
        self.assembler = assembler
        self.config = config
        self.linearSolver = config.linearSolver or LinearSolver()
        st = config.parameters._c()
        h = C.c_void_p()
        _err(lib().ikr_newton_create(C.byref(h), assembler.h, self.linearSolver.h, C.byref(st)), "newton")
        self.h = h
        self._cbs = []

    def __del__(self):
        if getattr(self, "h", None) and _lib is not None:
            _lib.ikr_newton_destroy(self.h)
            self.h = None

    def subscribe(self, fn):
        """fn(message: NonLinearSolverMessages, state: dict)"""
        def tramp(msg, st, _user):
            s = st.contents
            fn(NonLinearSolverMessages(msg), dict(residualNorm=s.residual_norm, correctionNorm=s.correction_norm,
                                                  iterations=s.iterations, loadFactor=s.load_factor))
        cb = _NR_OBS(tramp)
        self._cbs.append(cb)
        _err(lib().ikr_newton_subscribe(self.h, cb, None), "subscribe")

    def subscribe_fe_state(self, on=True):
        _err(lib().ikr_newton_subscribe_fe_state(self.h, int(on)))

    def graph_iterations(self):
        """Newton iterations run as one CUDA graph launch each since creation (NRSettings.step_graphs)."""
        n = C.c_int64()
        _err(lib().ikr_newton_graph_iterations(self.h, C.byref(n)))
        return n.value

    def residual(self):
        """residual() (newtonraphson.hh:260-268): f(req) -> force vector with the Full Dirichlet treatment."""
        nr = self

        def f(req):
            out = np.zeros(nr.assembler.size())
            _err(lib().ikr_newton_residual(nr.h, req.h, _ptr(out)), "residual")
            return out
        return f

    def jacobian(self):
        """jacobian() (newtonraphson.hh:270-280): f(req) -> tangent (scipy CSC, Full Dirichlet treatment)."""
        nr = self

        def f(req):
            _err(lib().ikr_newton_jacobian(nr.h, req.h), "jacobian")
            return nr.assembler.export_csc(DBCOption.Full)
        return f

    def updateFunction(self):
        """updateFunction() (newtonraphson.hh:282-287): f(req, dx) adds dx to the displacement (and re-imposes
        inhomogeneous Dirichlet values)."""
        nr = self

        def f(req, dx):
            d = np.ascontiguousarray(dx, dtype=np.float64)
            _err(lib().ikr_newton_update(nr.h, req.h, _ptr(d)), "update")
        return f

    def exclude_instances(self, mask=None):
        """Keep the instances whose mask entry is true out of the following batched solves (None clears)."""
        if mask is None:
            _err(lib().ikr_newton_exclude_instances(self.h, 0, None))
            return
        m = np.ascontiguousarray(np.asarray(mask, dtype=bool).astype(np.uint8))
        _err(lib().ikr_newton_exclude_instances(self.h, len(m), _ptr(m, C.c_uint8)))

    def instance_info(self):
        """(iterations, residual norms, status) per instance of the last batched solve; status 1 converged,
        -1 taken out after its elements inverted (det C <= 0), -2 taken out still above its tolerance after
        maxIter (the others go on), -3 kept out by exclude_instances, -4 taken out after its CG ran out of iterations
        (set_batched_take_out)."""
        n = self.assembler.fes.n_instances
        it = np.zeros(n, dtype=np.int32)
        rn = np.zeros(n)
        cv = np.zeros(n, dtype=np.int32)
        _err(lib().ikr_newton_instance_info(self.h, _ptr(it, C.c_int32), _ptr(rn), _ptr(cv, C.c_int32)))
        return it, rn, cv

    def instance_linear_iterations(self):
        """CG iterations per instance over the last batched solve."""
        out = np.zeros(self.assembler.fes.n_instances, dtype=np.int64)
        _err(lib().ikr_newton_instance_linear_iterations(self.h, _ptr(out, C.c_int64)))
        return out

    def set_batched_cg(self, variant=-1, first_chunk=0):
        """Batched solves: the CG runs as launches of first_chunk (0: 128), then doubling, iterations, re-planned
        over the instances still running; variant -1 lets the planner choose per launch, 0 row loop, 1 one row per
        thread, 2 / 3 / 5 four / eight / sixteen threads per row with the matrix in shared memory, 4 one instance per
        16-CTA cluster (FP32; vectors in distributed shared memory) -- where it fits, else 0."""
        _err(lib().ikr_newton_set_batched_cg(self.h, int(variant), int(first_chunk)))

    def set_batched_take_out(self, unsolved_linear=True):
        """Batched solves: an instance whose CG ends above its tolerance after linear_max_iter is taken out
        (status -4)."""
        _err(lib().ikr_newton_set_batched_take_out(self.h, int(bool(unsolved_linear))))

    def batched_cg_variant_launches(self):
        """Batched CG launches since creation per kernel variant 0..5."""
        out = np.zeros(6, dtype=np.int64)
        _err(lib().ikr_newton_batched_cg_variant_launches(self.h, _ptr(out, C.c_int64)))
        return out

    def batched_cg_launches(self):
        n = C.c_int64()
        _err(lib().ikr_newton_batched_cg_launches(self.h, C.byref(n)))
        return n.value

    def solve(self, req: FERequirements, stepSize: float = 0.0) -> NonLinearSolverInformation:
        info = _NRInfo()
        _err(lib().ikr_newton_solve(self.h, req.h, stepSize, C.byref(info)), "NewtonRaphson::solve")
        return NonLinearSolverInformation._from(info)


@dataclass
class ControlInformation:  # controlinfos.hh:22-32
    success: bool = False
    solverInfos: list = field(default_factory=list)
    totalIterations: int = 0
    totalLinearIterations: int = 0
    name: str = "Load Control"


class LoadControl:
    """LoadControl (loadcontrol.hh:58-113); creating it subscribes the element state update to the solver
    as ControlRoutineFactory::create does (controlroutinefactory.hh:38-48)."""

    def __init__(self, nonLinearSolver: NewtonRaphson, loadSteps: int, tbeginEnd=(0.0, 1.0)):
        self.nonLinearSolver = nonLinearSolver
        self.loadSteps = loadSteps
        h = C.c_void_p()
        _err(lib().ikr_load_control_create(C.byref(h), nonLinearSolver.h, loadSteps, tbeginEnd[0], tbeginEnd[1]),
             "load control")
        self.h = h
        self._cbs = []

    def __del__(self):
        if getattr(self, "h", None) and _lib is not None:
            _lib.ikr_load_control_destroy(self.h)
            self.h = None

    def subscribe(self, fn):
        """fn(message: ControlMessages, state: dict)"""
        def tramp(msg, st, _user):
            s = st.contents
            fn(ControlMessages(msg), dict(loadStep=s.load_step, stepSize=s.step_size, loadFactor=s.load_factor,
                                          totalIterations=s.total_iterations,
                                          name=s.name.decode() if s.name else ""))
        cb = _CTRL_OBS(tramp)
        self._cbs.append(cb)
        _err(lib().ikr_load_control_subscribe(self.h, cb, None), "subscribe")

    def set_escalation(self, solver: "NewtonRaphson" = None, req: "FERequirements" = None):
        """Batched runs: an instance this run's solver takes out in a load step is solved again from the state at the
        step's start by `solver` on `req` (a twin element set with the same instances, e.g. FP64) and stays there
        for the rest of the run; its displacement is copied into the run's requirement at every step end.  No
        arguments switch it off."""
        self._esc = (solver, req)
        _err(lib().ikr_load_control_set_escalation(self.h, solver.h if solver else None, req.h if req else None),
             "escalation")

    def set_escalation_concurrent(self, on=True):
        """Solve the instances escalated in earlier steps on a second host thread and stream while this run's solver
        does the step, or one after the other (the default: measured faster)."""
        _err(lib().ikr_load_control_set_escalation_concurrent(self.h, int(bool(on))))

    def instance_status(self):
        """Per instance: the status of the solver that holds it at the end of the last run (1 converged; -1, -2, -4
        taken out)."""
        n = self.nonLinearSolver.assembler.fes.n_instances
        st = np.zeros(n, dtype=np.int32)
        _err(lib().ikr_load_control_instance_status(self.h, n, _ptr(st, C.c_int32)))
        return st

    def escalated(self):
        """Per instance: escalated in the last run."""
        n = self.nonLinearSolver.assembler.fes.n_instances
        m = np.zeros(n, dtype=np.uint8)
        _err(lib().ikr_load_control_escalated(self.h, n, _ptr(m, C.c_uint8)))
        return m.astype(bool)

    def set_predictor(self, kind: int = 0, predictor: "LearnedPredictor" = None, params=None, record=False):
        """Newton predictor of every load step: 0 none (reference), 1 previous increment, 2 learned, 3 second-order
        extrapolation u + 2 du1 - du2 (2 and 3 fall back to the previous increment when their FP64 residual is not
        smaller)."""
        par = None if params is None else np.ascontiguousarray(params, dtype=np.float64)
        _err(lib().ikr_load_control_set_predictor(self.h, int(kind), predictor.h if predictor else None,
                                                  _ptr(par) if par is not None else None, int(record)), "predictor")

    def predictor_stats(self):
        a, r = C.c_int32(), C.c_int32()
        _err(lib().ikr_load_control_predictor_stats(self.h, C.byref(a), C.byref(r)))
        return a.value, r.value

    def set_predictor_gate(self, gated=True):
        """Keep the learned candidate only when its FP64 residual beats its fallback (default), or always."""
        _err(lib().ikr_load_control_set_predictor_gate(self.h, int(bool(gated))))

    def predictor_history(self):
        """Per load step of the last run: (step, |R| unpredicted, |R| previous increment, |R| learned, kept,
        |R| second-order extrapolation); kept: 0 unpredicted, 1 previous increment, 2 learned, 3 second-order
        (-1 where a candidate was not evaluated)."""
        n = C.c_int32()
        _err(lib().ikr_load_control_predictor_history(self.h, 0, None, C.byref(n)))
        out = np.zeros((max(n.value, 1), 6))
        _err(lib().ikr_load_control_predictor_history(self.h, n.value, _ptr(out), C.byref(n)))
        return out[:n.value]

    def run(self, req: FERequirements) -> ControlInformation:
        cap = self.loadSteps + 1
        infos = (_NRInfo * cap)()
        ci = _ControlInfo()
        _err(lib().ikr_load_control_run(self.h, req.h, C.byref(ci), infos, cap), "LoadControl::run")
        return ControlInformation(bool(ci.success), [NonLinearSolverInformation._from(infos[i])
                                                     for i in range(min(ci.n_solver_infos, cap))],
                                  ci.total_iterations, ci.total_linear_iterations)


class ArcLength:
    """Subsidiary function of the standard arc-length method (pathfollowingfunctions.hh:88-203)."""
    kind = 0

    def name(self):
        return "Arc length"


class LoadControlSubsidiaryFunction:
    """Subsidiary function f = Dlambda - s (pathfollowingfunctions.hh:217-281)."""
    kind = 1

    def name(self):
        return "Load Control"


class DisplacementControl:
    """Subsidiary function f = ||DD(controlledIndices)|| - s (pathfollowingfunctions.hh:295-368)."""
    kind = 2

    def __init__(self, controlledIndices):
        self.controlledIndices = [int(i) for i in controlledIndices]

    def name(self):
        return "Displacement Control"


class AdaptiveStepSizing:
    """AdaptiveStepSizing::NoOp and ::IterationBased (adaptivestepsizing.hh:14-57)."""

    class NoOp:
        kind = 0

        def targetIterations(self):
            return 0

    class IterationBased:
        kind = 1

        def __init__(self, targetIterations=0):
            self._t = int(targetIterations)

        def targetIterations(self):
            return self._t

        def setTargetIterations(self, t):
            if int(t) == 0:
                raise IkarusError(-3, "TargetIterations should not be equal to 0.")
            self._t = int(t)


class PathFollowing:
    """PathFollowing (pathfollowing.hh:148-236) with NewtonRaphsonWithSubsidiaryFunction: the Newton object
    supplies the assembler, the linear solver and the tolerances; the default subsidiary function is the arc
    length and the default step-size adaptation NoOp."""

    def __init__(self, nonLinearSolver: NewtonRaphson, steps: int, stepSize: float, pathFollowingType=None,
                 adaptiveStepSizing=None):
        self.nonLinearSolver = nonLinearSolver
        self.steps = steps
        self.pathFollowingType = pathFollowingType if pathFollowingType is not None else ArcLength()
        ci = getattr(self.pathFollowingType, "controlledIndices", None)
        arr = np.ascontiguousarray(ci if ci else [], dtype=np.int32)
        h = C.c_void_p()
        _err(lib().ikr_path_following_create(C.byref(h), nonLinearSolver.h, int(steps), float(stepSize),
                                             int(self.pathFollowingType.kind), len(arr),
                                             _ptr(arr, C.c_int32) if len(arr) else None), "path following")
        self.h = h
        self._cbs = []
        if adaptiveStepSizing is not None and adaptiveStepSizing.kind == 1:
            _err(lib().ikr_path_following_set_adaptive_step_sizing(self.h, 1, adaptiveStepSizing.targetIterations()),
                 "adaptive step sizing")

    def __del__(self):
        if getattr(self, "h", None) and _lib is not None:
            _lib.ikr_path_following_destroy(self.h)
            self.h = None

    def name(self):
        return "Path following with " + self.pathFollowingType.name()

    def subscribe(self, fn):
        """fn(message: ControlMessages, state: dict)"""
        def tramp(msg, st, _user):
            s = st.contents
            fn(ControlMessages(msg), dict(loadStep=s.load_step, stepSize=s.step_size, loadFactor=s.load_factor,
                                          totalIterations=s.total_iterations,
                                          name=s.name.decode() if s.name else ""))
        cb = _CTRL_OBS(tramp)
        self._cbs.append(cb)
        _err(lib().ikr_path_following_subscribe(self.h, cb, None), "subscribe")

    def subsidiary_args(self):
        """dict(stepSize, Dlambda, f, dfdDlambda, psi, currentStep) of the current state."""
        out = np.zeros(6)
        _err(lib().ikr_path_following_subsidiary_args(self.h, _ptr(out)))
        return dict(stepSize=out[0], Dlambda=out[1], f=out[2], dfdDlambda=out[3], psi=out[4],
                    currentStep=int(out[5]))

    def stats(self):
        """Last run: FP64 refinement sweeps of the initial prediction, its final relative residual, its CG
        iterations, load-column solves skipped by the warm start."""
        out = np.zeros(4)
        _err(lib().ikr_path_following_stats(self.h, _ptr(out)))
        return dict(prediction_sweeps=int(out[0]), prediction_rel_residual=out[1], prediction_cg=int(out[2]),
                    load_solves_skipped=int(out[3]))

    def set_warm_start(self, on=True):
        """Start the load column's CG from the previous Newton iteration's solution (default) or from zero."""
        _err(lib().ikr_path_following_set_warm_start(self.h, int(bool(on))))

    def increment(self, n):
        """SubsidiaryArgs::DD of the current step (n dofs)."""
        out = np.zeros(n)
        _err(lib().ikr_path_following_increment(self.h, _ptr(out)))
        return out

    def run(self, req: FERequirements) -> ControlInformation:
        cap = self.steps + 1
        infos = (_NRInfo * cap)()
        ci = _ControlInfo()
        _err(lib().ikr_path_following_run(self.h, req.h, C.byref(ci), infos, cap), "PathFollowing::run")
        return ControlInformation(bool(ci.success), [NonLinearSolverInformation._from(infos[i])
                                                     for i in range(min(ci.n_solver_infos, cap))],
                                  ci.total_iterations, ci.total_linear_iterations)


# ---- learned Newton predictor ------------------------------------------------------------------------------
class MLP:
    """Dense network with GELU hidden layers, BF16 weights and FP32 accumulation, trained on the GPU."""

    def __init__(self, n_in, width, depth, n_out, seed=0):
        h = C.c_void_p()
        _err(lib().ikr_mlp_create(C.byref(h), n_in, width, depth, n_out, seed), "mlp")
        self.h, self.n_in, self.width, self.depth, self.n_out = h, n_in, width, depth, n_out

    def __del__(self):
        if getattr(self, "h", None) and _lib is not None:
            _lib.ikr_mlp_destroy(self.h)
            self.h = None

    def num_params(self):
        n = C.c_int64()
        _err(lib().ikr_mlp_num_params(self.h, C.byref(n)))
        return n.value

    @property
    def params(self):
        out = np.zeros(self.num_params(), dtype=np.float32)
        _err(lib().ikr_mlp_get_params(self.h, _ptr(out, C.c_float)))
        return out

    @params.setter
    def params(self, p):
        p = np.ascontiguousarray(p, dtype=np.float32)
        _err(lib().ikr_mlp_set_params(self.h, _ptr(p, C.c_float)))

    def forward(self, x):
        x = np.ascontiguousarray(x, dtype=np.float32)
        y = np.zeros((x.shape[0], self.n_out), dtype=np.float32)
        _err(lib().ikr_mlp_forward(self.h, x.shape[0], _ptr(x, C.c_float), _ptr(y, C.c_float)), "forward")
        return y

    def loss_grad(self, x, t):
        x = np.ascontiguousarray(x, dtype=np.float32)
        t = np.ascontiguousarray(t, dtype=np.float32)
        loss = C.c_float()
        g = np.zeros(self.num_params(), dtype=np.float32)
        _err(lib().ikr_mlp_loss_grad(self.h, x.shape[0], _ptr(x, C.c_float), _ptr(t, C.c_float), C.byref(loss),
                                     _ptr(g, C.c_float)), "loss_grad")
        return loss.value, g

    def train(self, x, t, epochs, batch, lr, seed=0):
        x = np.ascontiguousarray(x, dtype=np.float32)
        t = np.ascontiguousarray(t, dtype=np.float32)
        loss = C.c_float()
        _err(lib().ikr_mlp_train(self.h, x.shape[0], _ptr(x, C.c_float), _ptr(t, C.c_float), epochs, batch, lr, seed,
                                 C.byref(loss)), "train")
        return loss.value


class LearnedPredictor:
    """POD basis of converged displacement increments + MLP over [load parameters, load factor, POD coordinates
    of the previous two increments] predicting the next increment (trained on the GPU)."""

    def __init__(self, fes: FiniteElements, n_params, n_modes=64, width=256, depth=4, capacity=4096, seed=0):
        h = C.c_void_p()
        _err(lib().ikr_predictor_create(C.byref(h), fes.h, n_params, n_modes, width, depth, capacity, seed),
             "predictor")
        self.h, self.fes, self.n_params = h, fes, n_params

    def __del__(self):
        if getattr(self, "h", None) and _lib is not None:
            _lib.ikr_predictor_destroy(self.h)
            self.h = None

    def num_snapshots(self):
        n = C.c_int64()
        _err(lib().ikr_predictor_num_snapshots(self.h, C.byref(n)))
        return n.value

    def fit(self, epochs=300, batch=128, lr=1e-3):
        loss, energy = C.c_float(), C.c_double()
        _err(lib().ikr_predictor_fit(self.h, epochs, batch, lr, C.byref(loss), C.byref(energy)), "fit")
        return loss.value, energy.value
