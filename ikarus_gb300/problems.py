"""Workload definitions: the cantilever and block problems the reference's tests and the benchmark configs use.

A ``Problem`` is plain data (mesh, NeoHooke parameters, EAS choice, Dirichlet flags, dead face tractions,
manipulator point loads, load stepping), so the same definition feeds the GPU path and the CPU oracle.
"""
from __future__ import annotations

from dataclasses import dataclass

import numpy as np

from .mesh import (HexMesh, boundary_faces, face_centers, fixed_dofs_where, jitter_interior, structured_hex_grid,
                   vertex_at)


def lame(E, nu):
    """(E, nu) -> (lambda, mu) (ikarus/finiteelements/physicshelper.hh:81-85, 123-127)."""
    return E * nu / ((1.0 + nu) * (1.0 - 2.0 * nu)), E / (2.0 * (1.0 + nu))


@dataclass
class Problem:
    name: str
    mesh: HexMesh
    lam: float
    mu: float
    eas: int = 0
    n_eas: int = 0
    fixed: np.ndarray = None
    face_elem: np.ndarray = None
    face_local: np.ndarray = None
    face_traction: np.ndarray = None  # per face, load factor 1
    pl_dofs: np.ndarray = None
    pl_values: np.ndarray = None
    load_steps: int = 10
    t_end: float = 1.0
    tol: float = 1e-10
    relative: bool = False
    material: int = 0  # 0 NeoHooke, 1 StVenantKirchhoff, 2 BlatzKo
    hyper: object = None  # a Hyperelastic law (the hyperelastic framework) instead of ``material``

    @property
    def n_dofs(self):
        return self.mesh.n_dofs


def cantilever_golden(eas: int, n_eas: int, nx=10, ny=1, nz=1, material=0) -> Problem:
    """tests/src/testcantileverbeam.hh:42-198 in 3D: YaspGrid 10x1x1 on (10, 2, 2), E = 100, nu = 0.3 (BlatzKo:
    mu = 40, testcantileverbeamEAS.cpp:101-104), clamped at x = 0, manipulator point loads R[y-dof] += lambda at
    the vertices (10,2,2) and (10,2,0), 20 load steps, ||R|| < 1e-10 (testcantileverbeamEAS.cpp:60-124)."""
    L, h = 10.0, 2.0
    m = structured_hex_grid(nx, ny, nz, (L, h, h))
    lam, mu = lame(100.0, 0.3) if material != 2 else (0.0, 40.0)
    fixed = fixed_dofs_where(m, lambda X: np.abs(X[:, 0]) < 1e-8)
    dofs = np.array([3 * vertex_at(m, (L, h, h)) + 1, 3 * vertex_at(m, (L, h, 0.0)) + 1], dtype=np.int32)
    return Problem(f"cantilever_golden_eas{eas}_{n_eas}", m, lam, mu, eas, n_eas, fixed, pl_dofs=dofs,
                   pl_values=np.ones(2), load_steps=20, tol=1e-10, material=material)


def cantilever(nx, ny, nz, L=10.0, E=1000.0, nu=0.3, jitter=0.0, seed=0, load_steps=10, traction=(0.0, 0.0, -1.0),
               eas=0, n_eas=0, tol=1e-10, relative=False) -> Problem:
    """Cantilever [0,L]x[0,1]x[0,1] clamped at x = 0 with a uniform dead traction on the face x = L."""
    m = structured_hex_grid(nx, ny, nz, (L, 1.0, 1.0))
    if jitter > 0:
        m = jitter_interior(m, jitter, seed)
    lam, mu = lame(E, nu)
    fixed = fixed_dofs_where(m, lambda X: np.abs(X[:, 0]) < 1e-8)
    fe, fl = boundary_faces(m, "x+")
    t = np.tile(np.asarray(traction, dtype=np.float64), (len(fe), 1))
    return Problem(f"cantilever_{nx}x{ny}x{nz}", m, lam, mu, eas, n_eas, fixed, fe, fl, t, load_steps=load_steps,
                   tol=tol, relative=relative)


def config1() -> Problem:
    """16x4x4 Q1 cantilever, E = 1000, nu = 0.3, traction (0,0,-1) on x = 10, 10 steps, ||R|| < 1e-10."""
    return cantilever(16, 4, 4, load_steps=10, tol=1e-10)


def config2(seed=2024, load_steps=20) -> Problem:
    """128x32x32 Q1 cantilever (131072 elements, 421443 dofs), interior vertices jittered by U(-0.1h, 0.1h),
    20 load steps, ||R||/||R0|| < 1e-8 per load step."""
    p = cantilever(128, 32, 32, jitter=0.1, seed=seed, load_steps=load_steps, tol=1e-8, relative=True)
    p.name = "cantilever_128x32x32_jittered"
    return p


def eas_block(nx=64, ny=64, nz=16, nu=0.4999, E=1000.0, pressure=50.0, load_steps=25, eas=1, n_eas=9) -> Problem:
    """Block [0,1]x[0,1]x[0,0.25], bottom face clamped, dead normal pressure on the centred 0.5 x 0.5 top patch,
    9-parameter EAS (nearly incompressible when nu = 0.4999)."""
    m = structured_hex_grid(nx, ny, nz, (1.0, 1.0, 0.25))
    lam, mu = lame(E, nu)
    fixed = fixed_dofs_where(m, lambda X: np.abs(X[:, 2]) < 1e-12)
    fe, fl = boundary_faces(m, "z+")
    c = face_centers(m, fe, fl)
    sel = (c[:, 0] > 0.25) & (c[:, 0] < 0.75) & (c[:, 1] > 0.25) & (c[:, 1] < 0.75)
    fe, fl = fe[sel], fl[sel]
    t = np.tile(np.array([0.0, 0.0, -pressure]), (len(fe), 1))
    return Problem(f"eas_block_{nx}x{ny}x{nz}", m, lam, mu, eas, n_eas, fixed, fe, fl, t, load_steps=load_steps,
                   tol=1e-8, relative=True)


def learned_cantilever(nx=64, ny=16, nz=16, L=10.0, E=1000.0, nu=0.3, load_steps=20) -> Problem:
    """Cantilever [0,L]x[0,1]x[0,1] clamped at x = 0 for the learned predictor; its loads come from
    ``learned_loads`` (distributed pressure on the top face z = 1 and a tip traction on x = L)."""
    m = structured_hex_grid(nx, ny, nz, (L, 1.0, 1.0))
    lam, mu = lame(E, nu)
    fixed = fixed_dofs_where(m, lambda X: np.abs(X[:, 0]) < 1e-8)
    p = Problem(f"learned_cantilever_{nx}x{ny}x{nz}", m, lam, mu, 0, 0, fixed, load_steps=load_steps, tol=1e-8,
                relative=True)
    return p


def sample_load_parameters(rng, n_modes=8, tip_max=2.0):
    """theta = (a_1..a_8, T): a_k ~ N(0, 0.5^2 / k), tip traction magnitude T ~ U[0, tip_max]."""
    a = rng.normal(0.0, 0.5 / np.sqrt(np.arange(1, n_modes + 1)))
    return np.concatenate([a, [rng.uniform(0.0, tip_max)]])


def learned_loads(p: Problem, theta):
    """Per-face dead tractions at load factor 1: top face pressure p(x) = sum_k a_k sin(k pi x / L) acting
    downwards, and the tip traction (0, 0, -T) on the face x = L.  Returns (face_elem, face_local, traction)."""
    L = p.mesh.lengths[0]
    fe_t, fl_t = boundary_faces(p.mesh, "z+")
    xc = face_centers(p.mesh, fe_t, fl_t)[:, 0]
    k = np.arange(1, len(theta))
    pres = np.sin(np.outer(xc, k) * np.pi / L) @ np.asarray(theta[:-1])
    t_top = np.zeros((len(fe_t), 3))
    t_top[:, 2] = -pres
    fe_x, fl_x = boundary_faces(p.mesh, "x+")
    t_tip = np.tile([0.0, 0.0, -float(theta[-1])], (len(fe_x), 1))
    return (np.concatenate([fe_t, fe_x]).astype(np.int32), np.concatenate([fl_t, fl_x]).astype(np.int32),
            np.concatenate([t_top, t_tip]))


@dataclass
class BatchedProblem:
    """Independent cantilevers concatenated into one mesh (disjoint node ranges)."""
    name: str
    mesh: HexMesh
    node_offsets: np.ndarray
    elem_offsets: np.ndarray
    lam_e: np.ndarray
    mu_e: np.ndarray
    fixed: np.ndarray
    face_elem: np.ndarray
    face_local: np.ndarray
    face_traction: np.ndarray
    parts: list  # per instance: Problem
    load_steps: int = 10

    @property
    def n_dofs(self):
        return self.mesh.n_dofs


def batched_cantilevers(n=512, seed=7, nx=(4, 32), nyz=(2, 8), L=(4.0, 12.0), E=(1e2, 1e4), nu=(0.2, 0.45),
                        t=(0.1, 2.0), load_steps=10) -> BatchedProblem:
    """n cantilevers [0,L]x[0,1]x[0,1] clamped at x = 0, each with a random grid nx x ny x nz, length, Young's
    modulus (log-uniform), Poisson ratio and a tip traction of random magnitude and direction on x = L."""
    rng = np.random.default_rng(seed)
    parts, coords, conns, lam_e, mu_e, fixed, fes, fls, trs = [], [], [], [], [], [], [], [], []
    noff, eoff = [0], [0]
    for i in range(n):
        gx = int(rng.integers(nx[0], nx[1] + 1))
        gy, gz = (int(v) for v in rng.integers(nyz[0], nyz[1] + 1, size=2))
        Li = float(rng.uniform(*L))
        Ei = float(np.exp(rng.uniform(np.log(E[0]), np.log(E[1]))))
        nui = float(rng.uniform(*nu))
        d = rng.standard_normal(3)
        d /= np.linalg.norm(d)
        tv = float(rng.uniform(*t)) * d
        p = cantilever(gx, gy, gz, L=Li, E=Ei, nu=nui, load_steps=load_steps, traction=tuple(tv), tol=1e-8,
                       relative=True)
        parts.append(p)
        coords.append(p.mesh.coords)
        conns.append(p.mesh.conn + noff[-1])
        lam_e.append(np.full(p.mesh.n_elems, p.lam))
        mu_e.append(np.full(p.mesh.n_elems, p.mu))
        fixed.append(p.fixed)
        fes.append(p.face_elem + eoff[-1])
        fls.append(p.face_local)
        trs.append(p.face_traction)
        noff.append(noff[-1] + p.mesh.n_nodes)
        eoff.append(eoff[-1] + p.mesh.n_elems)
    m = HexMesh(np.concatenate(coords), np.concatenate(conns).astype(np.int32))
    return BatchedProblem(f"batched_{n}_cantilevers", m, np.array(noff, dtype=np.int32), np.array(eoff),
                          np.concatenate(lam_e), np.concatenate(mu_e), np.concatenate(fixed),
                          np.concatenate(fes).astype(np.int32), np.concatenate(fls).astype(np.int32),
                          np.concatenate(trs), parts, load_steps)


def build_gpu_batched(bp: BatchedProblem, precision=1):
    from . import FiniteElements, NeoHooke, Precision, SparseFlatAssembler
    fes = FiniteElements(bp.mesh.coords, bp.mesh.conn, NeoHooke(1.0, 1.0))
    fes.set_element_materials(bp.lam_e, bp.mu_e)
    fes.set_instances(bp.node_offsets)
    fes.add_neumann(bp.face_elem, bp.face_local, bp.face_traction)
    return fes, SparseFlatAssembler(fes, bp.fixed, Precision(precision))


def single_element(offsets=None, E=1000.0, nu=0.3, eas=0, n_eas=0) -> Problem:
    """One hexahedron on the unit cube, corners moved by ``offsets`` (8 x 3) as in tests/src/testcommon.hh."""
    m = structured_hex_grid(1, 1, 1, (1.0, 1.0, 1.0))
    if offsets is not None:
        m.coords = m.coords + np.asarray(offsets, dtype=np.float64)
    lam, mu = lame(E, nu)
    return Problem("single_element", m, lam, mu, eas, n_eas, np.zeros(24, dtype=np.uint8))


def build_gpu(p: Problem, precision=0):
    """GPU objects for a problem: (FiniteElements, SparseFlatAssembler)."""
    from . import BlatzKo, FiniteElements, NeoHooke, Precision, SparseFlatAssembler, StVenantKirchhoff
    material = getattr(p, "material", 0)
    law = p.hyper if getattr(p, "hyper", None) is not None else {
        0: lambda: NeoHooke(p.lam, p.mu), 1: lambda: StVenantKirchhoff(p.lam, p.mu), 2: lambda: BlatzKo(p.mu)}[material]()
    fes = FiniteElements(p.mesh.coords, p.mesh.conn, law, p.eas, p.n_eas)
    if p.face_elem is not None and len(p.face_elem):
        fes.add_neumann(p.face_elem, p.face_local, p.face_traction)
    asm = SparseFlatAssembler(fes, p.fixed, Precision(precision))
    if p.pl_dofs is not None:
        asm.add_point_loads(p.pl_dofs, p.pl_values)
    return fes, asm
