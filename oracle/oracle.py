"""Python driver of the FP64 CPU oracle (test infrastructure only).

Wraps `oracle/pfem_oracle.cpp` (built into `oracle/build/liboracle.so`) and restates the
two control loops of the reference that sit above the element kernels:

* the PSPG Picard loop, `PicardAlgo::solve` (`srcs/simulation/nonLinearAlgo/PicardAlgo.cpp:31-95`)
  with the closures of `MomContEqIncompNewton::m_setupPicardPSPG`
  (`srcs/simulation/physics/IncompNewton/MomContEquationPSPG.inl:261-373`).  The linear solve
  is SuperLU with COLAMD column ordering (scipy.sparse.linalg.splu), standing in for Eigen 3.3's
  `SparseLU<SparseMatrix<double>, COLAMDOrdering<int>>` (a port of the same supernodal SuperLU
  algorithm; `MomContEquation.hpp:11`).  Eigen is not available here;
* the incompressible time loop, `SolverIncompNewton::m_solveIncompNewtonNoT` and
  `computeNextDT` (`srcs/simulation/physics/IncompNewton/Solver.cpp:216-247`), without the
  remesh.

Parity status: UNPINNED (the reference has no tests or golden vectors and cannot be built
here).  Only tests/, __graft_entry__.smoke() and bench.py's CPU legs may import this module.
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess
import sys
import time

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
SRC = os.path.join(HERE, "pfem_oracle.cpp")
LIB = os.path.join(HERE, "build", "liboracle.so")


def build(force=False):
    """Compile the oracle shared library (g++, OpenMP, no FMA contraction so x86 and Arm agree)."""
    if not force and os.path.exists(LIB) and os.path.getmtime(LIB) >= os.path.getmtime(SRC):
        return LIB
    os.makedirs(os.path.dirname(LIB), exist_ok=True)
    tmp = LIB + f".tmp{os.getpid()}"
    cmd = ["g++", "-O2", "-std=c++17", "-fopenmp", "-ffp-contract=off", "-fPIC", "-shared", SRC, "-o", tmp]
    subprocess.check_call(cmd)
    os.replace(tmp, LIB)
    return LIB


class PspgParams(C.Structure):
    _fields_ = [("rho", C.c_double), ("mu", C.c_double), ("dt", C.c_double), ("g", C.c_double * 3),
                ("gamma", C.c_double), ("tau0", C.c_double), ("mReg", C.c_double),
                ("alpha", C.c_double), ("Tr", C.c_double), ("T", C.POINTER(C.c_double)),
                ("dgammaDT", C.c_double)]


class HeatParams(C.Structure):
    _fields_ = [("rho", C.c_double), ("cv", C.c_double), ("k", C.c_double), ("h", C.c_double),
                ("Tinf", C.c_double), ("epsRad", C.c_double), ("fsFlags", C.c_int32), ("phaseChange", C.c_int32),
                ("Tm", C.c_double), ("DT", C.c_double), ("Lm", C.c_double)]


# heat boundary-condition flags (per node, and for the free-surface tag)
HT_T, HT_Q, HT_QH, HT_QR = 1, 2, 4, 8


class WcParams(C.Structure):
    _fields_ = [("K0", C.c_double), ("K0p", C.c_double), ("rhoStar", C.c_double), ("mu", C.c_double),
                ("g", C.c_double * 3), ("meduri", C.c_int), ("sc", C.c_double), ("maxDT", C.c_double),
                ("gamma", C.c_double), ("version", C.c_int)]


# SolverWCompNewton ids (WCompNewton/Solver.cpp:22-23): the continuity equation's unknown
WC_DPDT, WC_RHO, WC_DRHODT = 0, 1, 2


class FsParams(C.Structure):
    _fields_ = [("rho", C.c_double), ("mu", C.c_double), ("dt", C.c_double), ("gammaFS", C.c_double),
                ("g", C.c_double * 3), ("gamma", C.c_double)]


class WcBqParams(C.Structure):
    """Problem "BoussinesqWC": momentum and heat material of WCompNewton (MomEquation.inl:36-51,
    HeatEquation.inl:26-45)."""
    _fields_ = [("alpha", C.c_double), ("Tr", C.c_double), ("dgammaDT", C.c_double), ("phaseChange", C.c_int32),
                ("fsFlags", C.c_int32), ("C", C.c_double), ("eps", C.c_double), ("Tm", C.c_double), ("DT", C.c_double),
                ("Lm", C.c_double), ("k", C.c_double), ("cv", C.c_double), ("h", C.c_double), ("Tinf", C.c_double),
                ("epsRad", C.c_double)]


_lib = None


def lib():
    global _lib
    if _lib is None:
        build()
        L = C.CDLL(LIB)
        dp, ip, u8p, vp = C.POINTER(C.c_double), C.POINTER(C.c_int32), C.POINTER(C.c_uint8), C.c_void_p
        L.orc_create.restype = vp
        L.orc_create.argtypes = [C.c_int, C.c_int, dp, u8p, C.c_int, ip]
        L.orc_destroy.argtypes = [vp]
        L.orc_set_facets.restype = C.c_int
        L.orc_set_facets.argtypes = [vp, C.c_int, ip, ip]
        L.orc_surface_tension.argtypes = [vp, C.c_double, C.c_int, dp]
        L.orc_num_threads.restype = C.c_int
        L.orc_set_num_threads.argtypes = [C.c_int]
        for name in ("orc_get_positions", "orc_set_positions", "orc_update_positions_from_save",
                     "orc_update_positions"):
            getattr(L, name).argtypes = [vp, dp]
        L.orc_get_is_free.argtypes = [vp, u8p]
        L.orc_get_geometry.argtypes = [vp, dp, dp, dp]
        L.orc_save_nodes.argtypes = [vp]
        L.orc_restore_nodes.argtypes = [vp]
        L.orc_pspg_element.argtypes = [vp, C.c_int, C.POINTER(PspgParams), dp, dp, dp, dp]
        L.orc_pspg_assemble.restype = C.c_int
        L.orc_pspg_assemble.argtypes = [vp, C.POINTER(PspgParams), dp, dp, dp, C.c_int]
        L.orc_pspg_get.argtypes = [vp, ip, ip, dp, dp]
        L.orc_heat_assemble.restype = C.c_int
        L.orc_heat_assemble.argtypes = [vp, C.POINTER(HeatParams), C.c_double, dp, u8p, dp, dp, dp]
        L.orc_facet_gauss_positions.argtypes = [vp, dp]
        L.orc_wc_step.argtypes = [vp, C.POINTER(WcParams), C.c_double, dp, dp]
        L.orc_wc_next_dt.restype = C.c_double
        L.orc_wc_next_dt.argtypes = [vp, C.POINTER(WcParams), dp]
        L.orc_fs_build.argtypes = [vp, C.POINTER(FsParams), dp, dp, dp, u8p]
        L.orc_fs_pressure_rhs.argtypes = [vp, C.POINTER(FsParams), dp, dp, u8p]
        L.orc_fs_velocity_rhs.argtypes = [vp, C.POINTER(FsParams), dp]
        L.orc_fs_get.restype = C.c_int
        L.orc_fs_get.argtypes = [vp, C.c_int, ip, ip, dp, dp]
        L.orc_wc_bq_step.argtypes = [vp, C.POINTER(WcParams), C.POINTER(WcBqParams), C.c_double, dp, dp, u8p, dp, dp]
        L.orc_wc_bq_next_dt.restype = C.c_double
        L.orc_wc_bq_next_dt.argtypes = [vp, C.POINTER(WcParams), C.POINTER(WcBqParams), dp]
        L.orc_volume.restype = C.c_double
        L.orc_volume.argtypes = [vp]
        L.orc_wc_mass.restype = C.c_double
        L.orc_wc_mass.argtypes = [vp, dp]
        L.orc_tip.restype = C.c_double
        L.orc_tip.argtypes = [vp, C.c_int, C.c_int]
        _lib = L
    return _lib


def _dp(a):
    return a.ctypes.data_as(C.POINTER(C.c_double))


def _ip(a):
    return a.ctypes.data_as(C.POINTER(C.c_int32))


def set_threads(n):
    lib().orc_set_num_threads(int(n))


def num_threads():
    return lib().orc_num_threads()


class OracleMesh:
    """The reference's `Mesh` as far as the hot path uses it: node positions (with a saved
    copy), flags, connectivity and per-element J/detJ/invJ."""

    def __init__(self, mesh):
        self.dim, self.N, self.E = mesh.dim, mesh.n_nodes, mesh.n_elems
        self._pos = np.ascontiguousarray(mesh.pos, dtype=np.float64)
        self._flags = np.ascontiguousarray(mesh.flags, dtype=np.uint8)
        self._conn = np.ascontiguousarray(mesh.conn, dtype=np.int32)
        self.h = lib().orc_create(self.dim, self.N, _dp(self._pos),
                                  self._flags.ctypes.data_as(C.POINTER(C.c_uint8)), self.E, _ip(self._conn))
        if not self.h:
            raise ValueError("oracle: invalid mesh")
        facets = getattr(mesh, "facets", None)
        if facets is not None and facets.shape[1]:
            self.set_facets(facets, mesh.facet_elm)

    def set_facets(self, facets, facet_elm):
        self._facets = np.ascontiguousarray(facets, dtype=np.int32)
        self._facet_elm = np.ascontiguousarray(facet_elm, dtype=np.int32)
        if lib().orc_set_facets(self.h, self._facet_elm.size, _ip(self._facets), _ip(self._facet_elm)):
            raise ValueError("oracle: invalid facets")

    def surface_tension(self, gamma, any_node=True):
        """Surface tension forces alone (dim, N) at the current positions."""
        out = np.empty((self.dim, self.N))
        lib().orc_surface_tension(self.h, float(gamma), int(any_node), _dp(out))
        return out

    def __del__(self):
        if getattr(self, "h", None) and _lib is not None:
            _lib.orc_destroy(self.h)
            self.h = None

    @property
    def positions(self):
        out = np.empty((self.dim, self.N))
        lib().orc_get_positions(self.h, _dp(out))
        return out

    def set_positions(self, pos):
        pos = np.ascontiguousarray(pos, dtype=np.float64)
        lib().orc_set_positions(self.h, _dp(pos))

    def is_free(self):
        out = np.empty(self.N, np.uint8)
        lib().orc_get_is_free(self.h, out.ctypes.data_as(C.POINTER(C.c_uint8)))
        return out.astype(bool)

    def geometry(self):
        J = np.empty((self.E, 3, 3))
        inv = np.empty((self.E, 3, 3))
        det = np.empty(self.E)
        lib().orc_get_geometry(self.h, _dp(J), _dp(det), _dp(inv))
        return J, det, inv

    def save(self):
        lib().orc_save_nodes(self.h)

    def restore(self):
        lib().orc_restore_nodes(self.h)

    def update_from_save(self, delta):
        delta = np.ascontiguousarray(delta, dtype=np.float64)
        lib().orc_update_positions_from_save(self.h, _dp(delta))

    def volume(self):
        return lib().orc_volume(self.h)

    def tip(self, coord=0, want_max=True):
        return lib().orc_tip(self.h, coord, int(want_max))


def pspg_params(rho, mu, dt, g, gamma=0.0, tau0=0.0, m_reg=0.0, boussinesq=None):
    """boussinesq: None, or (alpha, Tr, T[, DgammaDT]) with T the node temperatures (kept alive on p)."""
    p = PspgParams()
    p.rho, p.mu, p.dt, p.gamma, p.tau0, p.mReg = rho, mu, dt, gamma, tau0, m_reg
    for i, x in enumerate(g):
        p.g[i] = x
    if boussinesq is not None:
        alpha, Tr, T = boussinesq[:3]
        p._T = np.ascontiguousarray(T, dtype=np.float64)
        p.alpha, p.Tr, p.T = alpha, Tr, _dp(p._T)
        p.dgammaDT = boussinesq[3] if len(boussinesq) > 3 else 0.0
    return p


def pspg_element(om, e, rho, mu, dt, g, q_iter, q_prev, tau0=0.0, m_reg=0.0):
    npe = om.dim + 1
    nt = (om.dim + 1) * npe
    Ae = np.empty((nt, nt))
    be = np.empty(nt)
    p = pspg_params(rho, mu, dt, g, tau0=tau0, m_reg=m_reg)
    lib().orc_pspg_element(om.h, e, C.byref(p), _dp(np.ascontiguousarray(q_iter, float)),
                           _dp(np.ascontiguousarray(q_prev, float)), _dp(Ae), _dp(be))
    return Ae, be


def pspg_assemble(om, rho, mu, dt, g, q_iter, q_prev, vbc=None, apply_bc=True, gamma=0.0, tau0=0.0, m_reg=0.0,
                  boussinesq=None):
    """A (scipy CSC, Eigen's storage order) and b of m_buildAbPSPG (+ m_applyBCPSPG)."""
    import scipy.sparse as sp

    R = (om.dim + 1) * om.N
    if vbc is None:
        vbc = np.zeros(om.dim * om.N)
    p = pspg_params(rho, mu, dt, g, gamma, tau0, m_reg, boussinesq)
    q_iter = np.ascontiguousarray(q_iter, float)
    q_prev = np.ascontiguousarray(q_prev, float)
    vbc = np.ascontiguousarray(vbc, float)
    nnz = lib().orc_pspg_assemble(om.h, C.byref(p), _dp(q_iter), _dp(q_prev), _dp(vbc), int(apply_bc))
    colptr = np.empty(R + 1, np.int32)
    rowidx = np.empty(nnz, np.int32)
    vals = np.empty(nnz)
    b = np.empty(R)
    lib().orc_pspg_get(om.h, _ip(colptr), _ip(rowidx), _dp(vals), _dp(b))
    return sp.csc_matrix((vals, rowidx, colptr), shape=(R, R)), b


class PicardResult:
    def __init__(self):
        self.converged = False
        self.iterations = 0
        self.residuals = []
        self.times = {}


def _tick(times, key, t0):
    times[key] = times.get(key, 0.0) + time.perf_counter() - t0


def pspg_picard_step(om, q_prev, dt, rho=1000.0, mu=1e-3, g=(0.0, -9.81), vbc=None, max_iter=10,
                     min_res=1e-6, times=None, gamma=0.0, tau0=0.0, m_reg=0.0, boussinesq=None):
    """One `MomContEqIncompNewton::solve` with PSPG (Picard, residual "Ax_f").

    Mutates the oracle mesh positions.  Returns (q, PicardResult); on failure the positions
    are restored and q is q_prev (the node states are restored with the node list in the
    reference, `Mesh::restoreNodesList`)."""
    from scipy.sparse.linalg import splu

    res = PicardResult()
    times = res.times if times is None else times
    g = tuple(g) + (0.0,) * (3 - len(g))
    q_prev = np.asarray(q_prev, float)
    # prepare (:264-277)
    t0 = time.perf_counter()
    om.save()
    _tick(times, "Save/restore nodelist", t0)
    t0 = time.perf_counter()
    A, b = pspg_assemble(om, rho, mu, dt, g, q_prev, q_prev, vbc, gamma=gamma, tau0=tau0, m_reg=m_reg,
                         boussinesq=boussinesq)
    _tick(times, "Compute triplets+Assemble matrix+Apply boundary conditions", t0)
    q_iter = np.zeros_like(q_prev)
    r = float("inf")
    it = 0
    while r > min_res:
        if it > max_iter:
            om.restore()
            res.iterations = it
            return q_prev.copy(), res
        # solve closure (:278-313)
        t0 = time.perf_counter()
        try:
            lu = splu(A, permc_spec="COLAMD")
        except RuntimeError:
            _tick(times, "Factorize A matrix", t0)
            om.restore()
            res.iterations = it
            return q_prev.copy(), res
        _tick(times, "Factorize A matrix", t0)
        t0 = time.perf_counter()
        q_iter = lu.solve(b)
        _tick(times, "Solve system", t0)
        t0 = time.perf_counter()
        om.update_from_save(q_iter * dt)
        _tick(times, "Update solutions", t0)
        t0 = time.perf_counter()
        A, b = pspg_assemble(om, rho, mu, dt, g, q_iter, q_prev, vbc, gamma=gamma, tau0=tau0, m_reg=m_reg,
                             boussinesq=boussinesq)
        _tick(times, "Compute triplets+Assemble matrix+Apply boundary conditions", t0)
        # residual closure, "Ax_f" (:366-371)
        t0 = time.perf_counter()
        r = float(np.linalg.norm(A @ q_iter - b))
        _tick(times, "Compute Picard Algo residual", t0)
        res.residuals.append(r)
        if np.isnan(r):
            om.restore()
            res.iterations = it + 1
            return q_prev.copy(), res
        it += 1
    res.converged = True
    res.iterations = it
    return q_iter, res


def fs_gauge(mesh):
    """Pressure gauge nodes of the fractional step: in every connected group of elements (two
    elements are connected when they share a node) its smallest free-surface node, or its
    smallest node when it has none."""
    import scipy.sparse as sp
    from scipy.sparse.csgraph import connected_components

    N, E, npe = mesh.n_nodes, mesh.n_elems, mesh.dim + 1
    conn = np.asarray(mesh.conn)
    gauge = np.zeros(N, np.uint8)
    if E == 0:
        return gauge
    rows = np.repeat(conn[0], npe - 1)
    cols = conn[1:].T.ravel()
    adj = sp.csr_matrix((np.ones(rows.size), (rows, cols)), shape=(N, N))
    _, lab = connected_components(adj, directed=False)
    used = np.zeros(N, bool)
    used[conn.ravel()] = True
    fs = (np.asarray(mesh.flags) & 2) != 0
    best = {}
    for n in np.flatnonzero(used):
        c = lab[n]
        key = (0 if fs[n] else 1, n)
        if c not in best or key < best[c]:
            best[c] = key
    for _, n in best.values():
        gauge[n] = 1
    return gauge


def _fs_system(om, which, R):
    import scipy.sparse as sp

    nnz = lib().orc_fs_get(om.h, which, None, None, None, None)
    colptr = np.empty(R + 1, np.int32)
    rowidx = np.empty(nnz, np.int32)
    vals = np.empty(nnz)
    b = np.empty(R)
    lib().orc_fs_get(om.h, which, _ip(colptr), _ip(rowidx), _dp(vals), _dp(b))
    return sp.csc_matrix((vals, rowidx, colptr), shape=(R, R)), b


def fracstep_picard_step(om, q_prev, dt, rho=1000.0, mu=1e-3, g=(0.0, -9.81), gamma_fs=1.0, vbc=None, max_iter=10,
                         min_res=1e-6, residual="U", gauge=None, gamma=0.0, mesh=None):
    """One `MomContEqIncompNewton::solve` with the fractional step (m_setupPicardFracStep,
    MomContEquationFracStep.inl:463-630): per Picard iteration the three SparseLU solves of
    the velocity prediction, the pressure (gauge nodes pinned, see fs_gauge) and the velocity
    correction, then the positions from the saved ones.  residual "U" or "U_P" (the relative
    change of the iterate over the non-free nodes; "Ax_f" is unsupported there).
    q_prev = [v (d x N), p (N)].  Returns (q, PicardResult); on failure q_prev and the saved
    positions."""
    from scipy.sparse.linalg import splu

    d, N = om.dim, om.N
    res = PicardResult()
    gg = tuple(g) + (0.0,) * (3 - len(g))
    p = FsParams()
    p.rho, p.mu, p.dt, p.gammaFS, p.gamma = rho, mu, dt, gamma_fs, gamma
    for i in range(3):
        p.g[i] = gg[i]
    q_prev = np.asarray(q_prev, float)
    v_prev = np.ascontiguousarray(q_prev[:d * N])
    p_prev = np.ascontiguousarray(q_prev[d * N:(d + 1) * N])
    if vbc is None:
        vbc = np.zeros(d * N)
    vbc = np.ascontiguousarray(vbc, float)
    if gauge is None:
        gauge = fs_gauge(mesh)
    gauge = np.ascontiguousarray(gauge, np.uint8)
    gp = gauge.ctypes.data_as(C.POINTER(C.c_uint8))
    free = om.is_free()
    om.save()
    q_it_prev = q_prev.copy()
    r = float("inf")
    it = 0
    while r > min_res:
        if it > max_iter:
            om.restore()
            res.iterations = it
            return q_prev.copy(), res
        lib().orc_fs_build(om.h, C.byref(p), _dp(v_prev), _dp(p_prev), _dp(vbc), gp)
        A, b = _fs_system(om, 0, d * N)
        try:
            v_t = splu(A, permc_spec="COLAMD").solve(b)
        except RuntimeError:
            om.restore()
            res.iterations = it
            return q_prev.copy(), res
        lib().orc_fs_pressure_rhs(om.h, C.byref(p), _dp(np.ascontiguousarray(v_t)), _dp(p_prev), gp)
        L, bp = _fs_system(om, 1, N)
        try:
            p_it = splu(L, permc_spec="COLAMD").solve(bp)
        except RuntimeError:
            om.restore()
            res.iterations = it
            return q_prev.copy(), res
        dP = np.ascontiguousarray(p_it - gamma_fs * p_prev)
        lib().orc_fs_velocity_rhs(om.h, C.byref(p), _dp(dP))
        M, bv = _fs_system(om, 2, d * N)
        try:
            dv = splu(M, permc_spec="COLAMD").solve(bv)
        except RuntimeError:
            om.restore()
            res.iterations = it
            return q_prev.copy(), res
        v_it = v_t + dv
        q_it = np.concatenate([v_it, p_it])
        om.update_from_save(v_it * dt)
        # residual closure (:568-629)
        nf = ~free
        num = sum(float(np.sum((v_it[f * N:(f + 1) * N][nf] - q_it_prev[f * N:(f + 1) * N][nf]) ** 2)) for f in range(d))
        den = sum(float(np.sum(q_it_prev[f * N:(f + 1) * N][nf] ** 2)) for f in range(d))
        r_v = np.finfo(float).max if den == 0 else np.sqrt(num / den)
        r_p = 0.0
        if residual == "U_P":
            pn = p_it[nf] - q_it_prev[d * N:][nf]
            den_p = float(np.sum(q_it_prev[d * N:][nf] ** 2))
            r_p = np.finfo(float).max if den_p == 0 else np.sqrt(float(np.sum(pn ** 2)) / den_p)
        r = max(r_v, r_p)
        res.residuals.append(r)
        q_it_prev = q_it
        if np.isnan(r):
            om.restore()
            res.iterations = it + 1
            return q_prev.copy(), res
        it += 1
    res.converged = True
    res.iterations = it
    return q_it_prev, res


def heat_params(rho, cv, k, h=0.0, t_inf=0.0, eps_rad=0.0, fs_flags=0, phase_change=None):
    """phase_change: None or (Tm, DT, Lm)."""
    p = HeatParams()
    p.rho, p.cv, p.k, p.h, p.Tinf, p.epsRad, p.fsFlags = rho, cv, k, h, t_inf, eps_rad, int(fs_flags)
    if phase_change is not None:
        p.phaseChange = 1
        p.Tm, p.DT, p.Lm = phase_change
    return p


def heat_assemble(om, params, dt, t_prev, flags, t_bc=None, q_gp=None, t_state=None):
    """A (scipy CSC) and b of HeatEqIncompNewton::m_buildAb + m_applyBC from T_prev, with the
    node states t_state (default T_prev) in the phase-change factor and the facet terms."""
    import scipy.sparse as sp

    N = om.N
    t_prev = np.ascontiguousarray(t_prev, float)
    flags = np.ascontiguousarray(flags, np.uint8)
    t_bc = np.ascontiguousarray(np.zeros(N) if t_bc is None else t_bc, float)
    qp = None if q_gp is None else np.ascontiguousarray(q_gp, float)
    ts = None if t_state is None else np.ascontiguousarray(t_state, float)
    nnz = lib().orc_heat_assemble(om.h, C.byref(params), float(dt), _dp(t_prev),
                                  flags.ctypes.data_as(C.POINTER(C.c_uint8)), _dp(t_bc),
                                  None if qp is None else _dp(qp), None if ts is None else _dp(ts))
    colptr = np.empty(N + 1, np.int32)
    rowidx = np.empty(nnz, np.int32)
    vals = np.empty(nnz)
    b = np.empty(N)
    lib().orc_pspg_get(om.h, _ip(colptr), _ip(rowidx), _dp(vals), _dp(b))
    return sp.csc_matrix((vals, rowidx, colptr), shape=(N, N)), b


def heat_step(om, params, dt, t_prev, flags, t_bc=None, q_gp=None, max_iter=10, min_res=1e-6, residual="T",
              result=None):
    """`HeatEqIncompNewton::solve` (HeatEquation.inl:216-224) through `PicardAlgo::solve`
    (PicardAlgo.cpp:31-95): without phase change one pass (runOnlyOnce, :195-196); with it,
    Picard iterations that rebuild A and b from the new node temperatures (:131-138) until the
    residual "T" (relative change over the non-free nodes, :153-180) or "Ax_f" (:182-185) is at
    most min_res, failing after max_iter + 1 passes.  Linear solves by SuperLU/COLAMD.  Returns
    the temperatures (t_prev on failure); `result`, a dict, receives converged / iterations."""
    from scipy.sparse.linalg import splu

    t_prev = np.asarray(t_prev, float)
    free = om.is_free()
    A, b = heat_assemble(om, params, dt, t_prev, flags, t_bc, q_gp)
    t_it_prev = t_prev.copy()
    res, it = float("inf"), 0
    ok = True
    while res > min_res:
        if it > max_iter:
            ok = False
            break
        t_it = splu(A, permc_spec="COLAMD").solve(b)
        if params.phaseChange:
            A, b = heat_assemble(om, params, dt, t_prev, flags, t_bc, q_gp, t_state=t_it)
        if residual == "T":
            num = float(np.sum((t_it - t_it_prev)[~free] ** 2))
            den = float(np.sum(t_it_prev[~free] ** 2))
            res = float("inf") if den == 0 else np.sqrt(num / den)
        else:
            res = float(np.linalg.norm(A @ t_it - b))
        t_it_prev = t_it
        if np.isnan(res):
            ok = False
            break
        it += 1
        if not params.phaseChange:
            break
    if result is not None:
        result.update(converged=ok, iterations=it, residual=res)
    return t_it if ok else t_prev.copy()


def facet_gauss_positions(om):
    """Facet::getPosFromGP at the heat Gauss points: (F, 3, dim)."""
    F = om._facet_elm.size
    out = np.empty((F, 3, om.dim))
    lib().orc_facet_gauss_positions(om.h, _dp(out))
    return out


def wc_params(K0=2.2e7, K0p=7.0, rho_star=1000.0, mu=1e-3, g=(0.0, -9.81), meduri=True, sc=0.3, max_dt=1e-3,
              gamma=0.0, version=WC_DPDT):
    p = WcParams()
    p.K0, p.K0p, p.rhoStar, p.mu = K0, K0p, rho_star, mu
    gg = tuple(g) + (0.0,) * (3 - len(g))
    for i in range(3):
        p.g[i] = gg[i]
    p.meduri = int(meduri)
    p.sc = sc
    p.maxDT = max_dt
    p.gamma = gamma
    p.version = int(version)
    return p


def wc_step(om, params, dt, states, vbc=None):
    """In-place WC explicit step (CDS_dpdt, CDS_rho or CDS_drhodt by params.version) on
    `states` (float64, (2d+2)*N)."""
    if vbc is None:
        vbc = np.zeros(om.dim * om.N)
    assert states.dtype == np.float64 and states.flags.c_contiguous
    lib().orc_wc_step(om.h, C.byref(params), float(dt), _dp(states), _dp(np.ascontiguousarray(vbc, float)))


def wc_next_dt(om, params, states):
    return lib().orc_wc_next_dt(om.h, C.byref(params), _dp(np.ascontiguousarray(states, float)))


def wc_bq_params(alpha, t_ref, k, cv, dgamma_dt=0.0, h=0.0, t_inf=0.0, eps_rad=0.0, fs_flags=0, phase_change=None):
    """phase_change: None or dict(C=, eps=, Tm=, DT=, Lm=)."""
    b = WcBqParams()
    b.alpha, b.Tr, b.dgammaDT = alpha, t_ref, dgamma_dt
    b.k, b.cv, b.h, b.Tinf, b.epsRad = k, cv, h, t_inf, eps_rad
    b.fsFlags = fs_flags
    if phase_change:
        b.phaseChange = 1
        b.C, b.eps, b.Tm, b.DT, b.Lm = (phase_change[k] for k in ("C", "eps", "Tm", "DT", "Lm"))
    return b


def wc_bq_step(om, params, bq, dt, states, flags, vbc=None, t_bc=None, q_gp=None):
    """In-place BoussinesqWC step on `states` (float64, (2d+3)*N: v, p, rho, a, T); flags: heat
    flags per node (HT_*), t_bc the T-Dirichlet values at t + dt, q_gp the Q flux at the facet
    Gauss points ((F, 3, d))."""
    N = om.N
    if vbc is None:
        vbc = np.zeros(om.dim * N)
    if t_bc is None:
        t_bc = np.zeros(N)
    assert states.dtype == np.float64 and states.flags.c_contiguous and states.size == (2 * om.dim + 3) * N
    q = _dp(np.ascontiguousarray(q_gp, float)) if q_gp is not None else None
    lib().orc_wc_bq_step(om.h, C.byref(params), C.byref(bq), float(dt), _dp(states),
                         _dp(np.ascontiguousarray(vbc, float)), np.ascontiguousarray(flags, np.uint8).ctypes.data_as(
                             C.POINTER(C.c_uint8)), _dp(np.ascontiguousarray(t_bc, float)), q)


def wc_bq_next_dt(om, params, bq, states):
    return lib().orc_wc_bq_next_dt(om.h, C.byref(params), C.byref(bq), _dp(np.ascontiguousarray(states, float)))


def wc_mass(om, states):
    return lib().orc_wc_mass(om.h, _dp(np.ascontiguousarray(states, float)))


if __name__ == "__main__":
    print(build(force="--force" in sys.argv))
