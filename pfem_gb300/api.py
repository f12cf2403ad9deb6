"""ctypes binding of the C ABI in include/pfem_gpu.h (libpfemgpu.so).

This is the thin host layer the tests and the benchmark drive; it holds no numerics.  There
is no fallback: if the library was not built, loading raises.
"""
from __future__ import annotations

import ctypes as C
import os

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "libpfemgpu.so")

PFG_OK = 0
ERRORS = {-1: "PFG_ERR_INVALID", -2: "PFG_ERR_CUDA", -3: "PFG_ERR_NOMEM", -4: "PFG_ERR_STATE",
          -5: "PFG_ERR_UNSUPPORTED", -6: "PFG_ERR_DEVICE"}

KIND_INCOMP_PSPG = 0
KIND_WC_CDS_DPDT = 1
PREC_FP64 = 0
PREC_MIXED = 1
LINSOLVE_BICGSTAB = 0
LINSOLVE_LU = 1
PC_BLOCK_JACOBI = 0
PC_MULTIGRID = 1
ASM_FP32 = 0
ASM_DOUBLE_FLOAT = 1
RES_AX_F, RES_U, RES_U_P, RES_T = 0, 1, 2, 3
# continuity forms of the weakly compressible solver (pfg_wc_version)
WC_DPDT, WC_RHO, WC_DRHODT = 0, 1, 2

NODE_BOUND, NODE_FREE_SURFACE, NODE_FIXED, NODE_DIRICHLET, NODE_FREE = 1, 2, 4, 8, 16

# every symbol include/pfem_gpu.h declares
EXPORTED = (
    "pfg_default_params", "pfg_create", "pfg_destroy", "pfg_last_error", "pfg_upload_mesh", "pfg_set_states",
    "pfg_get_states", "pfg_get_positions", "pfg_get_flags", "pfg_set_dirichlet", "pfg_picard_step",
    "pfg_wc_step", "pfg_next_dt", "pfg_set_time", "pfg_volume", "pfg_mass", "pfg_tip", "pfg_pspg_assemble",
    "pfg_get_csr", "pfg_get_geometry", "pfg_linear_solve", "pfg_version", "pfg_set_profiling",
    "pfg_get_phase_times", "pfg_reset_phase_times", "pfg_phase_name", "pfg_wc_step_async", "pfg_synchronize",
    "pfg_get_stream", "pfg_wc_next_dt_noalloc", "pfg_set_instances", "pfg_picard_step_batch", "pfg_device_bytes",
    "pfg_upload_facets", "pfg_set_positions", "pfg_get_spmv_pairs", "pfg_set_temperature",
    "pfg_get_temperature", "pfg_heat_set_bc", "pfg_heat_set_flux", "pfg_heat_step", "pfg_upload_mesh_remap",
    "pfg_wc_step_batch", "pfg_set_tuning", "pfg_get_tuning",
)
NUM_PHASES = 17


class Params(C.Structure):
    _fields_ = [
        ("dim", C.c_int32), ("kind", C.c_int32), ("precision", C.c_int32), ("linear_solver", C.c_int32),
        ("gravity", C.c_double * 3), ("mu", C.c_double),
        ("rho", C.c_double), ("picard_max_iter", C.c_int32), ("residual", C.c_int32),
        ("picard_min_res", C.c_double), ("krylov_max_iter", C.c_int32), ("refine_max_iter", C.c_int32),
        ("krylov_rel_tol", C.c_double), ("krylov_abs_tol", C.c_double),
        ("K0", C.c_double), ("K0p", C.c_double), ("rho_star", C.c_double), ("security_coeff", C.c_double),
        ("max_dt", C.c_double), ("meduri", C.c_int32), ("pad1", C.c_int32),
        ("hbm_budget_bytes", C.c_size_t),
        ("inner_rel_tol", C.c_double),
        ("gamma", C.c_double),
        ("preconditioner", C.c_int32), ("assembly", C.c_int32),
        ("tau0", C.c_double), ("m_reg", C.c_double),
        ("heat_k", C.c_double), ("heat_cv", C.c_double), ("heat_h", C.c_double), ("heat_t_inf", C.c_double),
        ("heat_eps_rad", C.c_double), ("heat_fs_flags", C.c_int32), ("boussinesq", C.c_int32),
        ("alpha_t", C.c_double), ("t_ref", C.c_double), ("dgamma_dt", C.c_double),
        ("heat_max_iter", C.c_int32), ("heat_residual", C.c_int32), ("heat_min_res", C.c_double),
        ("heat_phase_change", C.c_int32), ("pad3", C.c_int32), ("heat_tm", C.c_double), ("heat_dt_melt", C.c_double),
        ("heat_lm", C.c_double), ("ck_c", C.c_double), ("ck_eps", C.c_double),
        ("gamma_fs", C.c_double), ("frac_step", C.c_int32), ("fs_pressure_dirichlet", C.c_int32),
        ("wc_version", C.c_int32), ("pad4", C.c_int32),
    ]


# heat boundary-condition flags (pfg_heat_flag)
HEAT_T, HEAT_Q, HEAT_QH, HEAT_QR = 1, 2, 4, 8


class StepStatus(C.Structure):
    _fields_ = [("converged", C.c_int32), ("picard_iterations", C.c_int32), ("krylov_iterations", C.c_int32),
                ("steps_done", C.c_int32), ("residual", C.c_double), ("dt", C.c_double), ("time", C.c_double),
                ("fp64_solves", C.c_int32), ("pad0", C.c_int32)]


class Tuning(C.Structure):
    """pfg_tuning: launch shapes of the tunable mixed-form kernels (0 = keep)."""
    _fields_ = [("spmv_lanes", C.c_int32), ("pair_block", C.c_int32), ("elem_block", C.c_int32),
                ("res_block", C.c_int32), ("mg_lanes", C.c_int32)]


class PfgError(RuntimeError):
    pass


_lib = None


def load(path=LIB_PATH):
    """Load libpfemgpu.so (raises if it is missing: no CPU fallback exists)."""
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(path):
        raise PfgError(f"{path} not built; run pfem_gb300.build.build() (no CPU fallback exists)")
    L = C.CDLL(path)
    vp, dp, ip, i64p, u8p = C.c_void_p, C.POINTER(C.c_double), C.POINTER(C.c_int32), C.POINTER(C.c_int64), \
        C.POINTER(C.c_uint8)
    sig = {
        "pfg_default_params": ([C.c_int32, C.c_int32, C.POINTER(Params)], C.c_int),
        "pfg_create": ([C.POINTER(Params), C.POINTER(vp)], C.c_int),
        "pfg_destroy": ([vp], C.c_int),
        "pfg_last_error": ([vp], C.c_char_p),
        "pfg_upload_mesh": ([vp, C.c_int32, dp, u8p, C.c_int32, ip], C.c_int),
        "pfg_upload_facets": ([vp, C.c_int32, ip, ip], C.c_int),
        "pfg_set_states": ([vp, dp], C.c_int),
        "pfg_get_states": ([vp, dp], C.c_int),
        "pfg_set_positions": ([vp, dp], C.c_int),
        "pfg_get_positions": ([vp, dp], C.c_int),
        "pfg_get_flags": ([vp, u8p], C.c_int),
        "pfg_set_dirichlet": ([vp, C.c_int32, ip, dp], C.c_int),
        "pfg_picard_step": ([vp, C.c_double, C.POINTER(StepStatus)], C.c_int),
        "pfg_wc_step": ([vp, C.c_double, C.c_int32, C.POINTER(StepStatus)], C.c_int),
        "pfg_wc_step_batch": ([vp, C.c_double, C.c_int32, C.POINTER(StepStatus)], C.c_int),
        "pfg_next_dt": ([vp, dp], C.c_int),
        "pfg_set_time": ([vp, C.c_double, C.c_double], C.c_int),
        "pfg_volume": ([vp, dp], C.c_int),
        "pfg_mass": ([vp, dp], C.c_int),
        "pfg_tip": ([vp, C.c_int32, C.c_int32, dp], C.c_int),
        "pfg_pspg_assemble": ([vp, C.c_double, dp, dp, C.c_int32], C.c_int),
        "pfg_get_csr": ([vp, ip, i64p, i64p, ip, dp, dp], C.c_int),
        "pfg_get_geometry": ([vp, dp, dp], C.c_int),
        "pfg_linear_solve": ([vp, dp, ip, dp], C.c_int),
        "pfg_version": ([], C.c_char_p),
        "pfg_set_profiling": ([vp, C.c_int32], C.c_int),
        "pfg_get_phase_times": ([vp, dp, i64p], C.c_int),
        "pfg_reset_phase_times": ([vp], C.c_int),
        "pfg_get_spmv_pairs": ([vp, i64p], C.c_int),
        "pfg_set_tuning": ([vp, C.POINTER(Tuning)], C.c_int),
        "pfg_get_tuning": ([vp, C.POINTER(Tuning)], C.c_int),
        "pfg_set_temperature": ([vp, dp], C.c_int),
        "pfg_upload_mesh_remap": ([vp, C.c_int32, dp, u8p, C.c_int32, ip, ip, C.c_int32], C.c_int),
        "pfg_get_temperature": ([vp, dp], C.c_int),
        "pfg_heat_set_bc": ([vp, u8p, dp], C.c_int),
        "pfg_heat_set_flux": ([vp, dp], C.c_int),
        "pfg_heat_step": ([vp, C.c_double, C.POINTER(StepStatus)], C.c_int),
        "pfg_phase_name": ([C.c_int32], C.c_char_p),
        "pfg_wc_step_async": ([vp, C.c_double, C.c_int32], C.c_int),
        "pfg_synchronize": ([vp, C.POINTER(StepStatus)], C.c_int),
        "pfg_get_stream": ([vp, C.POINTER(vp)], C.c_int),
        "pfg_wc_next_dt_noalloc": ([C.POINTER(Params), C.c_int32, C.c_int32, vp, vp, vp, vp, vp], C.c_int),
        "pfg_set_instances": ([vp, C.c_int32, ip, dp, dp], C.c_int),
        "pfg_picard_step_batch": ([vp, dp, C.POINTER(StepStatus)], C.c_int),
        "pfg_device_bytes": ([vp, C.POINTER(C.c_size_t)], C.c_int),
    }
    for name, (args, res) in sig.items():
        f = getattr(L, name)
        f.argtypes = args
        f.restype = res
    _lib = L
    return L


def _dp(a):
    return a.ctypes.data_as(C.POINTER(C.c_double)) if a is not None else None


def _ip(a):
    return a.ctypes.data_as(C.POINTER(C.c_int32)) if a is not None else None


def default_params(kind, dim):
    p = Params()
    rc = load().pfg_default_params(kind, dim, C.byref(p))
    if rc:
        raise PfgError(f"pfg_default_params: {ERRORS.get(rc, rc)}")
    return p


class Context:
    """One library context (one CUDA stream, one mesh)."""

    def __init__(self, params: Params):
        self.L = load()
        self.params = params
        self.h = C.c_void_p()
        rc = self.L.pfg_create(C.byref(params), C.byref(self.h))
        if rc:
            raise PfgError(f"pfg_create failed: {ERRORS.get(rc, rc)}")
        self.dim = params.dim
        self.N = 0
        self.E = 0

    def close(self):
        if self.h:
            self.L.pfg_destroy(self.h)
            self.h = C.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def _check(self, rc, what):
        if rc:
            msg = self.L.pfg_last_error(self.h).decode()
            raise PfgError(f"{what}: {ERRORS.get(rc, rc)}: {msg}")

    @property
    def nstates(self):
        return (self.dim + 1) if self.params.kind == KIND_INCOMP_PSPG else (2 * self.dim + 2)

    def upload_mesh(self, mesh):
        pos = np.ascontiguousarray(mesh.pos, np.float64)
        flags = np.ascontiguousarray(mesh.flags, np.uint8)
        conn = np.ascontiguousarray(mesh.conn, np.int32)
        self._check(self.L.pfg_upload_mesh(self.h, pos.shape[1], _dp(pos), flags.ctypes.data_as(C.POINTER(C.c_uint8)),
                                           conn.shape[1], conn.ctypes.data_as(C.POINTER(C.c_int32))),
                    "pfg_upload_mesh")
        self.N, self.E = pos.shape[1], conn.shape[1]
        facets = getattr(mesh, "facets", None)
        if facets is not None and facets.shape[1]:
            self.upload_facets(facets, mesh.facet_elm)

    def upload_mesh_remap(self, mesh, origin):
        """Upload a remeshed domain keeping the node states (and temperatures) on the device:
        origin (N_new, w) from `remesh.remesh_map`."""
        pos = np.ascontiguousarray(mesh.pos, np.float64)
        flags = np.ascontiguousarray(mesh.flags, np.uint8)
        conn = np.ascontiguousarray(mesh.conn, np.int32)
        org = np.ascontiguousarray(origin, np.int32)
        assert org.ndim == 2 and org.shape[0] == pos.shape[1]
        self._check(self.L.pfg_upload_mesh_remap(self.h, pos.shape[1], _dp(pos),
                                                 flags.ctypes.data_as(C.POINTER(C.c_uint8)), conn.shape[1],
                                                 conn.ctypes.data_as(C.POINTER(C.c_int32)), _ip(org), org.shape[1]),
                    "pfg_upload_mesh_remap")
        self.N, self.E = pos.shape[1], conn.shape[1]
        facets = getattr(mesh, "facets", None)
        if facets is not None and facets.shape[1]:
            self.upload_facets(facets, mesh.facet_elm)

    def upload_facets(self, facets, facet_elm):
        """The mesh's boundary facets (dim x F nodes) and the element of each."""
        facets = np.ascontiguousarray(facets, np.int32)
        facet_elm = np.ascontiguousarray(facet_elm, np.int32)
        self._check(self.L.pfg_upload_facets(self.h, facet_elm.size, _ip(facets), _ip(facet_elm)),
                    "pfg_upload_facets")

    def set_states(self, s):
        s = np.ascontiguousarray(s, np.float64)
        assert s.size == self.nstates * self.N
        self._check(self.L.pfg_set_states(self.h, _dp(s)), "pfg_set_states")

    def get_states(self, out=None):
        if out is None:
            out = np.empty(self.nstates * self.N)
        assert out.dtype == np.float64 and out.flags.c_contiguous and out.size == self.nstates * self.N
        self._check(self.L.pfg_get_states(self.h, _dp(out)), "pfg_get_states")
        return out

    def get_positions(self):
        out = np.empty((self.dim, self.N))
        self._check(self.L.pfg_get_positions(self.h, _dp(out)), "pfg_get_positions")
        return out

    def set_positions(self, pos):
        """Replace the node positions (dim, N), keeping connectivity and states."""
        pos = np.ascontiguousarray(pos, np.float64)
        assert pos.size == self.dim * self.N
        self._check(self.L.pfg_set_positions(self.h, _dp(pos)), "pfg_set_positions")

    def get_flags(self):
        out = np.empty(self.N, np.uint8)
        self._check(self.L.pfg_get_flags(self.h, out.ctypes.data_as(C.POINTER(C.c_uint8))), "pfg_get_flags")
        return out

    def set_dirichlet(self, nodes, values):
        nodes = np.ascontiguousarray(nodes, np.int32)
        values = np.ascontiguousarray(values, np.float64)
        self._check(self.L.pfg_set_dirichlet(self.h, nodes.size, nodes.ctypes.data_as(C.POINTER(C.c_int32)),
                                             _dp(values)), "pfg_set_dirichlet")

    # ---- heat equation (incompressible contexts) ----
    def set_temperature(self, T):
        T = np.ascontiguousarray(T, np.float64)
        assert T.size == self.N
        self._check(self.L.pfg_set_temperature(self.h, _dp(T)), "pfg_set_temperature")

    def get_temperature(self, out=None):
        if out is None:
            out = np.empty(self.N)
        assert out.dtype == np.float64 and out.flags.c_contiguous and out.size == self.N
        self._check(self.L.pfg_get_temperature(self.h, _dp(out)), "pfg_get_temperature")
        return out

    def heat_set_bc(self, flags, t_dirichlet=None):
        """Per-node heat BC flags (HEAT_T / HEAT_Q / HEAT_QH / HEAT_QR) and Dirichlet temperatures."""
        flags = np.ascontiguousarray(flags, np.uint8)
        assert flags.size == self.N
        tp = None
        if t_dirichlet is not None:
            self._tbc = np.ascontiguousarray(t_dirichlet, np.float64)
            assert self._tbc.size == self.N
            tp = _dp(self._tbc)
        self._check(self.L.pfg_heat_set_bc(self.h, flags.ctypes.data_as(C.POINTER(C.c_uint8)), tp),
                    "pfg_heat_set_bc")

    def heat_set_flux(self, q_gp):
        """Flux vectors at the three Gauss points of every facet, (F, 3, dim), or None."""
        if q_gp is None:
            self._check(self.L.pfg_heat_set_flux(self.h, None), "pfg_heat_set_flux")
            return
        q = np.ascontiguousarray(q_gp, np.float64)
        self._check(self.L.pfg_heat_set_flux(self.h, _dp(q)), "pfg_heat_set_flux")

    def heat_step(self, dt):
        st = StepStatus()
        self._check(self.L.pfg_heat_step(self.h, float(dt), C.byref(st)), "pfg_heat_step")
        return st

    def picard_step(self, dt):
        st = StepStatus()
        self._check(self.L.pfg_picard_step(self.h, float(dt), C.byref(st)), "pfg_picard_step")
        return st

    def device_bytes(self):
        """Device memory held by this context."""
        b = C.c_size_t()
        self._check(self.L.pfg_device_bytes(self.h, C.byref(b)), "pfg_device_bytes")
        return b.value

    def set_instances(self, node_offsets, rho, mu):
        """Declare the uploaded mesh a union of independent instances (mixed precision)."""
        off = np.ascontiguousarray(node_offsets, np.int32)
        n = len(off) - 1
        rho = np.ascontiguousarray(np.broadcast_to(np.asarray(rho, float), (n,)))
        mu = np.ascontiguousarray(np.broadcast_to(np.asarray(mu, float), (n,)))
        self._check(self.L.pfg_set_instances(self.h, n, _ip(off), _dp(rho), _dp(mu)), "pfg_set_instances")
        self.n_inst = n

    def picard_step_batch(self, dt):
        """One Picard step of every instance; returns one StepStatus per instance."""
        n = getattr(self, "n_inst", 1)
        dts = np.ascontiguousarray(np.broadcast_to(np.asarray(dt, float), (n,)))
        st = (StepStatus * n)()
        self._check(self.L.pfg_picard_step_batch(self.h, _dp(dts), st), "pfg_picard_step_batch")
        return list(st)

    def wc_step(self, dt, nsteps=1):
        st = StepStatus()
        self._check(self.L.pfg_wc_step(self.h, float(dt), int(nsteps), C.byref(st)), "pfg_wc_step")
        return st

    def wc_step_batch(self, dt, nsteps=1):
        """nsteps weakly compressible steps of every instance; one StepStatus per instance."""
        n = getattr(self, "n_inst", 1)
        st = (StepStatus * n)()
        self._check(self.L.pfg_wc_step_batch(self.h, float(dt), int(nsteps), st), "pfg_wc_step_batch")
        return list(st)

    def wc_step_async(self, dt, nsteps=1):
        self._check(self.L.pfg_wc_step_async(self.h, float(dt), int(nsteps)), "pfg_wc_step_async")

    def synchronize(self):
        st = StepStatus()
        self._check(self.L.pfg_synchronize(self.h, C.byref(st)), "pfg_synchronize")
        return st

    @property
    def stream(self):
        s = C.c_void_p()
        self._check(self.L.pfg_get_stream(self.h, C.byref(s)), "pfg_get_stream")
        return s.value or 0

    def next_dt(self):
        v = C.c_double()
        self._check(self.L.pfg_next_dt(self.h, C.byref(v)), "pfg_next_dt")
        return v.value

    def set_time(self, t, next_dt):
        self._check(self.L.pfg_set_time(self.h, float(t), float(next_dt)), "pfg_set_time")

    def volume(self):
        v = C.c_double()
        self._check(self.L.pfg_volume(self.h, C.byref(v)), "pfg_volume")
        return v.value

    def mass(self):
        v = C.c_double()
        self._check(self.L.pfg_mass(self.h, C.byref(v)), "pfg_mass")
        return v.value

    def tip(self, coord=0, want_max=True):
        v = C.c_double()
        self._check(self.L.pfg_tip(self.h, coord, int(want_max), C.byref(v)), "pfg_tip")
        return v.value

    def pspg_assemble(self, dt, q_iter=None, q_prev=None, apply_bc=True):
        qi = None if q_iter is None else np.ascontiguousarray(q_iter, np.float64)
        qp = None if q_prev is None else np.ascontiguousarray(q_prev, np.float64)
        self._check(self.L.pfg_pspg_assemble(self.h, float(dt), _dp(qi), _dp(qp), int(apply_bc)),
                    "pfg_pspg_assemble")

    def get_csr(self, values=True):
        nr = C.c_int32()
        nnz = C.c_int64()
        self._check(self.L.pfg_get_csr(self.h, C.byref(nr), C.byref(nnz), None, None, None, None), "pfg_get_csr")
        rp = np.empty(nr.value + 1, np.int64)
        ci = np.empty(nnz.value, np.int32)
        va = np.empty(nnz.value) if values else None
        b = np.empty(nr.value) if values else None
        self._check(self.L.pfg_get_csr(self.h, None, None, rp.ctypes.data_as(C.POINTER(C.c_int64)),
                                       ci.ctypes.data_as(C.POINTER(C.c_int32)), _dp(va), _dp(b)), "pfg_get_csr")
        return rp, ci, va, b

    def get_geometry(self):
        det = np.empty(self.E)
        inv = np.empty((self.E, 3, 3))
        self._check(self.L.pfg_get_geometry(self.h, _dp(det), _dp(inv)), "pfg_get_geometry")
        return det, inv

    def set_profiling(self, enable=True):
        self._check(self.L.pfg_set_profiling(self.h, int(enable)), "pfg_set_profiling")

    def reset_phase_times(self):
        self._check(self.L.pfg_reset_phase_times(self.h), "pfg_reset_phase_times")

    def phase_times(self):
        """{phase name: (total ms, launches)} for phases that ran."""
        ms = np.zeros(NUM_PHASES)
        n = np.zeros(NUM_PHASES, np.int64)
        self._check(self.L.pfg_get_phase_times(self.h, _dp(ms), n.ctypes.data_as(C.POINTER(C.c_int64))),
                    "pfg_get_phase_times")
        return {self.L.pfg_phase_name(i).decode(): (float(ms[i]), int(n[i])) for i in range(NUM_PHASES) if n[i]}

    def set_tuning(self, spmv_lanes=0, pair_block=0, elem_block=0, res_block=0, mg_lanes=0):
        t = Tuning(spmv_lanes, pair_block, elem_block, res_block, mg_lanes)
        self._check(self.L.pfg_set_tuning(self.h, C.byref(t)), "pfg_set_tuning")

    def get_tuning(self):
        t = Tuning()
        self._check(self.L.pfg_get_tuning(self.h, C.byref(t)), "pfg_get_tuning")
        return {k: int(getattr(t, k)) for k, _ in Tuning._fields_}

    def spmv_pairs(self):
        """Node pairs read by the timed Krylov SpMV launches since the last reset."""
        v = C.c_int64()
        self._check(self.L.pfg_get_spmv_pairs(self.h, C.byref(v)), "pfg_get_spmv_pairs")
        return int(v.value)

    def linear_solve(self, x0):
        x = np.ascontiguousarray(x0, np.float64).copy()
        it = C.c_int32()
        res = C.c_double()
        self._check(self.L.pfg_linear_solve(self.h, _dp(x), C.byref(it), C.byref(res)), "pfg_linear_solve")
        return x, it.value, res.value
