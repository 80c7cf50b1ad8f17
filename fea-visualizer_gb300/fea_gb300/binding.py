"""ctypes binding of libfea_gb300.so (include/fea_gpu.h).

`CUDASolver` mirrors the reference's solver interface (include/FEM/Solver.hpp:8-14:
advance_time / clear_values / has_numerical_instability) over the C ABI, with
the FEMContext inputs (mesh, boundary condition, equation parameters) passed
at construction.  There is no CPU fallback: constructing a solver without the
CUDA library or without a GPU raises.
"""
from __future__ import annotations

import ctypes as C
import os

import numpy as np

_PKG = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
LIB_PATH = os.path.join(_PKG, "lib", "libfea_gb300.so")

HEAT, WAVE, ADVECTION_DIFFUSION, REACTION_DIFFUSION = 0, 1, 2, 3
DIRICHLET, NEUMANN = 0, 1
FP32, FP64 = 0, 1
STIFFNESS, MASS, ADVECTION = 0, 1, 2

STATUS_BLOWUP, STATUS_NONFINITE, STATUS_NOT_CONVERGED, STATUS_BREAKDOWN = 1, 2, 4, 8
MESH_OPEN, MESH_CLOSED, MESH_MIRRORED = 0, 1, 2

ERRORS = {
    -1: "invalid argument", -2: "CUDA error", -3: "no CUDA device", -4: "bad mesh",
    -5: "out of memory", -6: "bad call order", -7: "unsupported", -8: "too large", -9: "solve failed",
}


class FeaError(RuntimeError):
    def __init__(self, code, msg):
        super().__init__(f"{ERRORS.get(code, code)}: {msg}")
        self.code = code


class Params(C.Structure):
    """fea_params (include/fea_gpu.h)."""
    _fields_ = [
        ("equation", C.c_int),
        ("heat_time_step", C.c_float), ("heat_conductivity", C.c_float),
        ("advdiff_time_step", C.c_float), ("advdiff_c", C.c_float), ("advdiff_velocity", C.c_float * 3),
        ("wave_time_step", C.c_float), ("wave_c", C.c_float),
        ("rd_time_step", C.c_float), ("rd_Du", C.c_float), ("rd_Dv", C.c_float),
        ("rd_feed_rate", C.c_float), ("rd_kill_rate", C.c_float),
        ("reaction_mode", C.c_int), ("wave_scheme", C.c_int),
        ("newmark_beta", C.c_double), ("newmark_gamma", C.c_double),
        ("advection_scheme", C.c_int), ("advection_sign", C.c_float), ("velocity_mode", C.c_int),
        ("cg_tolerance", C.c_double), ("cg_max_iterations", C.c_int), ("cg_refine", C.c_int),
        ("cg_initial_guess", C.c_int),
    ]


class Info(C.Structure):
    _fields_ = [
        ("num_vertices", C.c_int64), ("num_triangles", C.c_int64), ("num_boundary_points", C.c_int64),
        ("num_unknowns", C.c_int64), ("nnz", C.c_int64), ("max_row_nonzeros", C.c_int64),
        ("precision", C.c_int), ("boundary_condition", C.c_int), ("rows_per_warp_lanes", C.c_int),
        ("device_bytes", C.c_int64),
    ]


class Status(C.Structure):
    _fields_ = [
        ("flags", C.c_uint32), ("last_iterations", C.c_int32 * 2),
        ("last_rel_residual", C.c_double * 2), ("steps_done", C.c_int64), ("total_iterations", C.c_int64),
        ("cg_launches", C.c_int64),
    ]


class InstanceDesc(C.Structure):
    _fields_ = [
        ("vertices", C.c_void_p), ("num_vertices", C.c_int64),
        ("triangles", C.c_void_p), ("num_triangles", C.c_int64),
        ("boundary_condition", C.c_int),
        ("time_step", C.c_float), ("Du", C.c_float), ("Dv", C.c_float),
        ("feed_rate", C.c_float), ("kill_rate", C.c_float),
    ]


# every function of include/fea_gpu.h with its argument types
_P = C.c_void_p

# CG iteration kernel variants of fea_set_cg_variant, and those that finish
# each iteration at the start of the next launch (deferred finish)
CG_VARIANTS = (0, 1, 2, 3, 6, 7, 10, 11, 13, 14, 15, 4, 8, 16)
DEFERRED_VARIANTS = (10, 11, 13, 14, 15)
_I64 = C.c_int64
SIGNATURES = {
    "fea_params_default": [C.POINTER(Params)],
    "fea_create": [_P, _I64, _P, _I64, _P, C.c_int, C.c_int, C.POINTER(Params), C.POINTER(C.c_void_p)],
    "fea_destroy": [_P],
    "fea_set_boundary_condition": [_P, C.c_int],
    "fea_set_params": [_P, C.POINTER(Params)],
    "fea_set_element_fields": [_P, _P, _P],
    "fea_clear_values": [_P],
    "fea_set_values": [_P, _P],
    "fea_get_values": [_P, _P],
    "fea_set_fields": [_P, _P, _P],
    "fea_get_fields": [_P, _P, _P],
    "fea_set_fields_device": [_P, _P, _P],
    "fea_get_fields_device": [_P, _P, _P],
    "fea_advance_time": [_P, _I64],
    "fea_synchronize": [_P],
    "fea_has_numerical_instability": [_P, C.POINTER(C.c_int)],
    "fea_get_status": [_P, C.POINTER(Status)],
    "fea_get_info": [_P, C.POINTER(Info)],
    "fea_get_matrix": [_P, C.c_int, _P, _P, _P, _P],
    "fea_get_idx_map": [_P, _P, _P],
    "fea_autotune": [_P],
    "fea_set_cg_variant": [_P, C.c_int],
    "fea_get_stream": [_P, C.POINTER(C.c_void_p)],
    "fea_time_spmv": [_P, C.c_int, C.c_int, C.POINTER(C.c_double)],
    "fea_adjoint_advdiff": [_P, _P, _P, _I64, _I64, C.POINTER(C.c_double), _P, _P],
    "fea_adjoint_advdiff_device": [_P, _P, _P, _I64, _I64, C.POINTER(C.c_double), _P, _P],
    "fea_set_element_diffusivity_device": [_P, _P],
    "fea_adjoint_gray_scott": [_P, _P, _P, _P, _P, _I64, _I64, C.POINTER(C.c_double), _P, _P, _P],
    "fea_adjoint_gray_scott_device": [_P, _P, _P, _P, _P, _I64, _I64, C.POINTER(C.c_double), _P, _P, _P],
    "fea_smooth_normals": [_P, _P, C.c_float, _P],
    "fea_smooth_normals_device": [_P, _P, C.c_float, _P],
    "fea_export_ply": [_P, C.c_char_p, _P, C.c_float, C.c_float, C.c_int, _P],
    "fea_ply_geometry": [_P, _P, C.c_float, C.c_float, C.c_int, _P, _P, _I64, _P, _I64, C.POINTER(C.c_int64),
                         C.POINTER(C.c_int64)],
    "fea_batch_create": [C.POINTER(InstanceDesc), C.c_int, C.c_int, C.c_double, C.c_int, C.POINTER(C.c_void_p)],
    "fea_batch_destroy": [_P],
    "fea_batch_set_fields": [_P, C.c_int, _P, _P],
    "fea_batch_get_fields": [_P, C.c_int, _P, _P],
    "fea_batch_advance_time": [_P, _I64],
    "fea_batch_synchronize": [_P],
    "fea_batch_get_status": [_P, _P, _P],
    "fea_batch_set_cg": [_P, C.c_double, C.c_int],
    "fea_batch_get_counters": [_P, _P, _P],
    "fea_batch_time_iteration": [_P, C.c_int, C.POINTER(C.c_double)],
    "fea_batch_cg_variant": [_P, C.c_int, C.POINTER(C.c_int)],
    "fea_batch_set_initial_guess": [_P, C.c_int],
    "fea_pcg_solve_csr_noalloc": [_I64, _P, _P, _P, _P, _P, C.c_int, C.c_double, C.c_int, _P,
                                  C.POINTER(C.c_int), C.POINTER(C.c_double), C.POINTER(C.c_uint32)],
    "fea_triangulate_pslg": [_P, _I64, _P, _I64, _P, _I64, C.c_double, C.c_double, C.POINTER(C.c_void_p)],
    "fea_pslg_mesh_sizes": [_P, C.POINTER(_I64), C.POINTER(_I64)],
    "fea_pslg_mesh_copy": [_P, _P, _P, _P],
    "fea_pslg_mesh_destroy": [_P],
}

_lib = None


def load(path: str = LIB_PATH):
    """Load the library (raises if it has not been built)."""
    global _lib
    if _lib is None:
        if not os.path.exists(path):
            raise FeaError(-3, f"{path} is missing: build it with fea-visualizer_gb300/build.py")
        L = C.CDLL(path)
        for name, argt in SIGNATURES.items():
            f = getattr(L, name)
            f.argtypes = argt
            f.restype = C.c_int
        L.fea_last_error.restype = C.c_char_p
        L.fea_last_error.argtypes = []
        L.fea_version.restype = C.c_char_p
        L.fea_version.argtypes = []
        _lib = L
    return _lib


def check(rc):
    if rc != 0:
        raise FeaError(rc, load().fea_last_error().decode())
    return rc


def _ptr(a):
    return None if a is None else C.c_void_p(a.ctypes.data)


def default_params(**kw) -> Params:
    """EquationParameters.hpp defaults, then keyword overrides."""
    p = Params()
    check(load().fea_params_default(C.byref(p)))
    for k, v in kw.items():
        if k == "advdiff_velocity":
            p.advdiff_velocity[:] = list(v)
        else:
            setattr(p, k, v)
    return p


class CUDASolver:
    """The reference's Solver interface over the C ABI (one mesh, one GPU)."""

    def __init__(self, vertices, triangles, boundary_condition=DIRICHLET, precision=FP32, params=None,
                 on_boundary=None):
        L = load()
        self.vertices = np.ascontiguousarray(vertices, dtype=np.float32).reshape(-1, 3)
        self.triangles = np.ascontiguousarray(triangles, dtype=np.uint32).reshape(-1, 3)
        ob = None if on_boundary is None else np.ascontiguousarray(on_boundary, dtype=np.uint8)
        self.params = params if params is not None else default_params()
        self.precision = precision
        self.real = np.float64 if precision == FP64 else np.float32
        h = C.c_void_p()
        check(L.fea_create(_ptr(self.vertices), self.vertices.shape[0], _ptr(self.triangles),
                           self.triangles.shape[0], _ptr(ob), boundary_condition, precision,
                           C.byref(self.params), C.byref(h)))
        self._h = h

    # -- Solver.hpp:8-14 ---------------------------------------------------------
    def advance_time(self, nsteps: int = 1):
        check(load().fea_advance_time(self._h, int(nsteps)))

    def clear_values(self):
        check(load().fea_clear_values(self._h))

    def has_numerical_instability(self) -> bool:
        out = C.c_int(0)
        check(load().fea_has_numerical_instability(self._h, C.byref(out)))
        return bool(out.value)

    # -- FEMContext-side inputs ---------------------------------------------------
    def set_params(self, params: Params):
        self.params = params
        check(load().fea_set_params(self._h, C.byref(params)))

    def set_boundary_condition(self, bc: int):
        check(load().fea_set_boundary_condition(self._h, bc))

    def set_element_fields(self, diffusivity=None, velocity=None):
        d = None if diffusivity is None else np.ascontiguousarray(diffusivity, dtype=np.float32)
        v = None if velocity is None else np.ascontiguousarray(velocity, dtype=np.float32)
        check(load().fea_set_element_fields(self._h, _ptr(d), _ptr(v)))

    # -- fields -------------------------------------------------------------------
    @property
    def info(self) -> Info:
        i = Info()
        check(load().fea_get_info(self._h, C.byref(i)))
        return i

    def status(self) -> Status:
        s = Status()
        check(load().fea_get_status(self._h, C.byref(s)))
        return s

    def set_values(self, values):
        v = np.ascontiguousarray(values, dtype=np.float32)
        check(load().fea_set_values(self._h, _ptr(v)))

    def get_values(self):
        out = np.zeros(self.vertices.shape[0], dtype=np.float32)
        check(load().fea_get_values(self._h, _ptr(out)))
        return out

    def set_fields(self, u=None, v=None):
        uu = None if u is None else np.ascontiguousarray(u, dtype=np.float32)
        vv = None if v is None else np.ascontiguousarray(v, dtype=np.float32)
        check(load().fea_set_fields(self._h, _ptr(uu), _ptr(vv)))

    def get_fields(self):
        u = np.zeros(self.vertices.shape[0], dtype=np.float32)
        v = np.zeros(self.vertices.shape[0], dtype=np.float32)
        check(load().fea_get_fields(self._h, _ptr(u), _ptr(v)))
        return u, v

    def set_fields_device(self, u_ptr, v_ptr):
        check(load().fea_set_fields_device(self._h, u_ptr, v_ptr))

    def get_fields_device(self, u_ptr, v_ptr):
        check(load().fea_get_fields_device(self._h, u_ptr, v_ptr))

    def synchronize(self):
        check(load().fea_synchronize(self._h))

    def autotune(self):
        check(load().fea_autotune(self._h))
        return self.info.rows_per_warp_lanes

    def set_cg_variant(self, variant: int):
        """0, 1: tile-ELL kernels (8 or 4 entries prefetched); 2, 3: tile-ELL streamed by bulk copies
        (2 or 3 stages); 6, 7: the same with two block barriers per tile; 10, 11: variants 2 and 7
        with the deferred finish (each launch finishes the previous one's iteration); 13: tile-ELL
        with direct loads pipelined one tile ahead, deferred finish; 14, 15: direct row loads with
        the operator in a ring of 3 or 4 bulk-copy stages, deferred finish; 4, 8, 16: windowed CSR
        kernels.  `CG_VARIANTS` lists them all."""
        check(load().fea_set_cg_variant(self._h, int(variant)))

    def stream(self) -> int:
        """cudaStream_t of the handle, as an integer."""
        st = C.c_void_p()
        check(load().fea_get_stream(self._h, C.byref(st)))
        return st.value or 0

    def time_spmv(self, reps=20, flush_l2=True) -> float:
        ms = C.c_double(0)
        check(load().fea_time_spmv(self._h, int(reps), 1 if flush_l2 else 0, C.byref(ms)))
        return ms.value

    def matrix(self, which):
        """(row_ptr, col, values, present) of K / M / Adv."""
        inf = self.info
        rp = np.zeros(inf.num_unknowns + 1, dtype=np.int32)
        col = np.zeros(inf.nnz, dtype=np.int32)
        val = np.zeros(inf.nnz, dtype=self.real)
        pres = np.zeros(inf.nnz, dtype=np.uint8)
        check(load().fea_get_matrix(self._h, which, _ptr(rp), _ptr(col), _ptr(val), _ptr(pres)))
        return rp, col, val, pres

    def idx_map(self):
        idx = np.zeros(self.vertices.shape[0], dtype=np.int32)
        ob = np.zeros(self.vertices.shape[0], dtype=np.uint8)
        check(load().fea_get_idx_map(self._h, _ptr(idx), _ptr(ob)))
        return idx, ob

    def adjoint_advdiff(self, u0, target, nsteps, checkpoint_every, grads=True):
        """(J, dJ/du0 node-indexed, dJ/dD per element) of the explicit advection-diffusion loss
        (gradients None when grads is False: forward and loss only)."""
        u0 = np.ascontiguousarray(u0, dtype=np.float32)
        tg = np.ascontiguousarray(target, dtype=np.float32)
        gu = np.zeros(self.vertices.shape[0], dtype=np.float32) if grads else None
        gd = np.zeros(self.triangles.shape[0], dtype=np.float32) if grads else None
        J = C.c_double(0)
        check(load().fea_adjoint_advdiff(self._h, _ptr(u0), _ptr(tg), int(nsteps), int(checkpoint_every),
                                         C.byref(J), _ptr(gu), _ptr(gd)))
        return J.value, gu, gd

    def adjoint_advdiff_device(self, u0, target, nsteps, checkpoint_every, grads=True):
        """The same on CUDA tensors: u0 and target unknown-indexed [N] in the handle's precision;
        returns (J, dJ/du0 [N], dJ/dD [T]) as tensors on the same device (None without grads)."""
        import torch
        dt = torch.float64 if self.precision == FP64 else torch.float32
        u0 = u0.detach().to(dtype=dt).contiguous()
        tg = target.detach().to(dtype=dt, device=u0.device).contiguous()
        gu = torch.zeros_like(u0) if grads else None
        gd = torch.zeros(self.triangles.shape[0], dtype=dt, device=u0.device) if grads else None
        J = C.c_double(0)
        torch.cuda.synchronize(u0.device)
        check(load().fea_adjoint_advdiff_device(self._h, u0.data_ptr(), tg.data_ptr(), int(nsteps),
                                                int(checkpoint_every), C.byref(J),
                                                gu.data_ptr() if grads else None, gd.data_ptr() if grads else None))
        return J.value, gu, gd

    def adjoint_gray_scott_device(self, u0, v0, target_u, target_v, nsteps, checkpoint_every, grads=True):
        """Gray-Scott adjoint on CUDA tensors (unknown-indexed [N], handle precision; a None target drops
        its loss term) -> (J, dJ/du0, dJ/dv0, numpy [dJ/dF, dJ/dk, dJ/dDu, dJ/dDv]); gradients None
        without grads."""
        import torch
        dt = torch.float64 if self.precision == FP64 else torch.float32
        u0 = u0.detach().to(dtype=dt).contiguous()
        v0 = v0.detach().to(dtype=dt, device=u0.device).contiguous()
        tu = None if target_u is None else target_u.detach().to(dtype=dt, device=u0.device).contiguous()
        tv = None if target_v is None else target_v.detach().to(dtype=dt, device=u0.device).contiguous()
        gu = torch.zeros_like(u0) if grads else None
        gv = torch.zeros_like(u0) if grads else None
        gp = np.zeros(4) if grads else None
        J = C.c_double(0)
        torch.cuda.synchronize(u0.device)
        check(load().fea_adjoint_gray_scott_device(
            self._h, u0.data_ptr(), v0.data_ptr(), None if tu is None else tu.data_ptr(),
            None if tv is None else tv.data_ptr(), int(nsteps), int(checkpoint_every), C.byref(J),
            gu.data_ptr() if grads else None, gv.data_ptr() if grads else None, _ptr(gp)))
        return J.value, gu, gv, gp

    def set_element_diffusivity_device(self, D):
        """Per-element diffusivity from a CUDA tensor [T] (handle precision)."""
        import torch
        dt = torch.float64 if self.precision == FP64 else torch.float32
        D = D.detach().to(dtype=dt).contiguous()
        torch.cuda.synchronize(D.device)
        check(load().fea_set_element_diffusivity_device(self._h, D.data_ptr()))

    # -- after the solve (Surface::calculate_normals, Surface::export_to_ply) -----
    def smooth_normals(self, normals, vertex_extrusion):
        """Extruded smooth normals of the displayed field -> float32[V, 3] (unnormalised)."""
        n = np.ascontiguousarray(normals, dtype=np.float32).reshape(-1, 3)
        out = np.zeros_like(n)
        check(load().fea_smooth_normals(self._h, _ptr(n), float(vertex_extrusion), _ptr(out)))
        return out

    def ply_geometry(self, normals, vertex_extrusion=0.25, threshold=0.0, mesh_type=MESH_OPEN):
        """(positions float32[n, 3], values float32[n], triangles uint32[m, 3]) of the clipped export."""
        n = np.ascontiguousarray(normals, dtype=np.float32).reshape(-1, 3)
        nv, nt = C.c_int64(0), C.c_int64(0)
        args = (float(vertex_extrusion), float(threshold), int(mesh_type))
        check(load().fea_ply_geometry(self._h, _ptr(n), *args, None, None, 0, None, 0, C.byref(nv), C.byref(nt)))
        pos = np.zeros((nv.value, 3), dtype=np.float32)
        val = np.zeros(nv.value, dtype=np.float32)
        tri = np.zeros((nt.value, 3), dtype=np.uint32)
        check(load().fea_ply_geometry(self._h, _ptr(n), *args, _ptr(pos), _ptr(val), nv.value, _ptr(tri), nt.value,
                                      C.byref(nv), C.byref(nt)))
        return pos, val, tri

    def export_ply(self, path, normals, vertex_extrusion=0.25, threshold=0.0, mesh_type=MESH_OPEN,
                   color_coeffs=None):
        """Surface::export_to_ply of the displayed field (color_coeffs: 7 RGB polynomial coefficients)."""
        n = np.ascontiguousarray(normals, dtype=np.float32).reshape(-1, 3)
        cc = None if color_coeffs is None else np.ascontiguousarray(color_coeffs, dtype=np.float32).reshape(21)
        check(load().fea_export_ply(self._h, os.fsencode(path), _ptr(n), float(vertex_extrusion), float(threshold),
                                    int(mesh_type), _ptr(cc)))

    def close(self):
        if getattr(self, "_h", None):
            load().fea_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


class BatchSolver:
    """Many Gray-Scott instances stepped together (fea_batch_* of include/fea_gpu.h).

    instances: sequence of dicts with keys vertices, triangles, and optionally
    boundary_condition (NEUMANN), time_step, Du, Dv, feed_rate, kill_rate.
    Each instance follows the mass-weighted Gray-Scott step of one mesh."""

    def __init__(self, instances, precision=FP32, cg_tolerance=0.0, cg_max_iterations=0):
        L = load()
        self._keep = []
        descs = (InstanceDesc * len(instances))()
        self.num_vertices = []
        for d, spec in zip(descs, instances):
            v = np.ascontiguousarray(spec["vertices"], dtype=np.float32).reshape(-1, 3)
            t = np.ascontiguousarray(spec["triangles"], dtype=np.uint32).reshape(-1, 3)
            self._keep += [v, t]
            d.vertices, d.num_vertices = v.ctypes.data, v.shape[0]
            d.triangles, d.num_triangles = t.ctypes.data, t.shape[0]
            d.boundary_condition = spec.get("boundary_condition", NEUMANN)
            d.time_step = spec.get("time_step", 0.001)
            d.Du = spec.get("Du", 0.08)
            d.Dv = spec.get("Dv", 0.04)
            d.feed_rate = spec.get("feed_rate", 0.035)
            d.kill_rate = spec.get("kill_rate", 0.06)
            self.num_vertices.append(v.shape[0])
        h = C.c_void_p()
        check(L.fea_batch_create(descs, len(instances), precision, float(cg_tolerance), int(cg_max_iterations),
                                 C.byref(h)))
        self._keep = []
        self._h = h
        self.num_instances = len(instances)

    def set_fields(self, i, u=None, v=None):
        uu = None if u is None else np.ascontiguousarray(u, dtype=np.float32)
        vv = None if v is None else np.ascontiguousarray(v, dtype=np.float32)
        check(load().fea_batch_set_fields(self._h, int(i), _ptr(uu), _ptr(vv)))

    def get_fields(self, i):
        if not 0 <= int(i) < self.num_instances:  # the library reports the bad index
            check(load().fea_batch_get_fields(self._h, int(i), None, None))
        n = self.num_vertices[i]
        u = np.zeros(n, dtype=np.float32)
        v = np.zeros(n, dtype=np.float32)
        check(load().fea_batch_get_fields(self._h, int(i), _ptr(u), _ptr(v)))
        return u, v

    def advance_time(self, nsteps: int = 1):
        check(load().fea_batch_advance_time(self._h, int(nsteps)))

    def synchronize(self):
        check(load().fea_batch_synchronize(self._h))

    @property
    def cg_variant(self) -> int:
        v = C.c_int(0)
        check(load().fea_batch_cg_variant(self._h, 0, C.byref(v)))
        return v.value

    def set_cg_variant(self, variant: int):
        """0, 1: tile-ELL kernels (8 or 4 entries prefetched); 4, 8: windowed CSR kernels;
        14: tile-ELL with the operator streamed through a bulk-copy ring."""
        v = C.c_int(int(variant))
        check(load().fea_batch_cg_variant(self._h, 1, C.byref(v)))

    def set_cg(self, tolerance: float, max_iterations: int = 0):
        """New CG stopping rule of every instance (fea_batch_set_cg)."""
        check(load().fea_batch_set_cg(self._h, float(tolerance), int(max_iterations)))

    def set_initial_guess(self, rule: int):
        """Start of the solves: 0 the state x_n, 1 the extrapolated 2 x_n - x_(n-1)
        (variant 14; fea_batch_set_initial_guess)."""
        check(load().fea_batch_set_initial_guess(self._h, int(rule)))

    def time_iteration(self, reps: int = 10) -> float:
        """ms per CG iteration launch over every instance (fea_batch_time_iteration)."""
        ms = C.c_double(0)
        check(load().fea_batch_time_iteration(self._h, int(reps), C.byref(ms)))
        return ms.value

    def counters(self):
        """(total CG iterations int64[n], steps done int64[n]) since creation."""
        it = np.zeros(self.num_instances, dtype=np.int64)
        st = np.zeros(self.num_instances, dtype=np.int64)
        check(load().fea_batch_get_counters(self._h, _ptr(it), _ptr(st)))
        return it, st

    def status(self):
        """(flags uint32[n], iterations int32[n, 2] of the last solve)."""
        f = np.zeros(self.num_instances, dtype=np.uint32)
        it = np.zeros((self.num_instances, 2), dtype=np.int32)
        check(load().fea_batch_get_status(self._h, _ptr(f), _ptr(it)))
        return f, it

    def close(self):
        if getattr(self, "_h", None):
            load().fea_batch_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def triangulate_pslg(points, segments, holes=None, max_area=0.005, min_angle=20.0):
    """Quality triangulation of a PSLG on the XZ plane (fea_triangulate_pslg):
    points (x, z) [P, 2], segments [S, 2] point indices, holes (x, z) [H, 2].
    Returns (vertices float32 [V, 3] as (x, 0, z), triangles uint32 [T, 3],
    on_boundary uint8 [V]), the inputs of CUDASolver (Surface::init_from_PSLG)."""
    L = load()
    pts = np.ascontiguousarray(points, dtype=np.float64).reshape(-1, 2)
    seg = np.ascontiguousarray(segments, dtype=np.int32).reshape(-1, 2)
    hol = None if holes is None or len(holes) == 0 else np.ascontiguousarray(holes, dtype=np.float64).reshape(-1, 2)
    h = C.c_void_p()
    check(L.fea_triangulate_pslg(_ptr(pts), pts.shape[0], _ptr(seg), seg.shape[0], _ptr(hol),
                                 0 if hol is None else hol.shape[0], float(max_area), float(min_angle), C.byref(h)))
    try:
        nv, nt = _I64(0), _I64(0)
        check(L.fea_pslg_mesh_sizes(h, C.byref(nv), C.byref(nt)))
        xyz = np.zeros((nv.value, 3), dtype=np.float32)
        tri = np.zeros((nt.value, 3), dtype=np.uint32)
        ob = np.zeros(nv.value, dtype=np.uint8)
        check(L.fea_pslg_mesh_copy(h, _ptr(xyz), _ptr(tri), _ptr(ob)))
    finally:
        L.fea_pslg_mesh_destroy(h)
    return xyz, tri, ob
