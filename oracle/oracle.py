"""ctypes front end of the CPU restatement in this folder.

TEST INFRASTRUCTURE ONLY: imported by tests/, `__graft_entry__.smoke()` and the
CPU-baseline leg of bench.py, as the checker.  The product never imports it.

Parity status: unpinned against reference outputs (the reference has no golden
vectors and needs Eigen/glm, which are absent); pinned against derived
known-answer tests in tests/test_oracle.py.  Every function names the
reference code it restates (paths relative to the reference project).
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
_LIB_PATH = os.path.join(_HERE, "_build", "libfea_oracle.so")
_lib = None

HEAT, WAVE, ADVECTION_DIFFUSION, REACTION_DIFFUSION = 0, 1, 2, 3
DIRICHLET, NEUMANN = 0, 1


class Params(C.Structure):
    """Mirror of fo_params (oracle/fea_oracle.h)."""
    _fields_ = [
        ("equation", C.c_int), ("dt", C.c_double), ("kappa", C.c_double),
        ("Du", C.c_double), ("Dv", C.c_double), ("F", C.c_double), ("k", C.c_double),
        ("reaction_mode", C.c_int), ("wave_scheme", C.c_int),
        ("beta", C.c_double), ("gamma", C.c_double),
        ("adv_scheme", C.c_int), ("adv_sign", C.c_double), ("k_scaled", C.c_int),
        ("tol", C.c_double), ("max_iter", C.c_int), ("warm_start", C.c_int),
        ("nthreads", C.c_int), ("prev_u", C.c_void_p), ("prev_v", C.c_void_p),
    ]


def build(force: bool = False) -> str:
    """Compile the restatement with its Makefile (gcc, no other dependency)."""
    srcs = [f for f in os.listdir(_HERE) if f.endswith((".c", ".h"))]
    stale = not os.path.exists(_LIB_PATH) or any(
        os.path.getmtime(os.path.join(_HERE, f)) > os.path.getmtime(_LIB_PATH) for f in srcs)
    if force or stale:
        subprocess.run(["make", "-s", "-C", _HERE], check=True)
    return _LIB_PATH


def lib():
    global _lib
    if _lib is None:
        build()
        L = C.CDLL(_LIB_PATH)
        p = C.c_void_p
        i64 = C.c_int64
        L.fo_boundary.restype = i64
        L.fo_boundary.argtypes = [i64, i64, p, p]
        L.fo_idx_map.restype = i64
        L.fo_idx_map.argtypes = [i64, p, C.c_int, p]
        L.fo_pattern_build.restype = p
        L.fo_pattern_build.argtypes = [i64, i64, p, p, p, C.c_int]
        L.fo_pattern_nnz.restype = i64
        L.fo_pattern_nnz.argtypes = [p]
        L.fo_pattern_rows.restype = i64
        L.fo_pattern_rows.argtypes = [p]
        L.fo_pattern_copy.restype = None
        L.fo_pattern_copy.argtypes = [p, p, p, p, p]
        L.fo_pattern_free.restype = None
        L.fo_pattern_free.argtypes = [p]
        for s in ("f64", "f32"):
            f = getattr(L, f"fo_element_matrices_{s}")
            f.restype = None
            f.argtypes = [i64, p, p, C.c_int, p, p, p, p, p]
            f = getattr(L, f"fo_sum_{s}")
            f.restype = None
            f.argtypes = [i64, p, p, p, i64, p]
            f = getattr(L, f"fo_spmv_{s}")
            f.restype = None
            f.argtypes = [i64, p, p, p, p, p]
            f = getattr(L, f"fo_pcg_{s}")
            f.restype = i64
            f.argtypes = [i64, p, p, p, p, p, C.c_double, i64, C.c_int, C.c_int, C.POINTER(C.c_double)]
            f = getattr(L, f"fo_step_{s}")
            f.restype = i64
            f.argtypes = [i64, p, p, p, p, p, C.POINTER(Params), p, p, p, i64, C.POINTER(i64)]
            f = getattr(L, f"fo_newmark_init_{s}")
            f.restype = C.c_int
            f.argtypes = [i64, p, p, p, p, C.POINTER(Params), p, p]
            f = getattr(L, f"fo_instability_{s}")
            f.restype = C.c_int
            f.argtypes = [i64, p, p]
        L.fo_adjoint_gray_scott_f64.restype = C.c_double
        L.fo_adjoint_gray_scott_f64.argtypes = [i64, p, p, p, p, C.POINTER(Params), p, p, p, p, i64, i64, p, p, p]
        L.fo_smooth_normals_f32.restype = None
        L.fo_smooth_normals_f32.argtypes = [i64, i64, p, p, p, p, C.c_float, p]
        L.fo_ply_clip.restype = i64
        L.fo_ply_clip.argtypes = [i64, i64, p, p, p, p, C.c_float, C.c_float, C.c_int, p, p, i64, p, i64,
                                  C.POINTER(C.c_int64)]
        L.fo_adjoint_advdiff_f64.restype = C.c_double
        L.fo_adjoint_advdiff_f64.argtypes = [i64, i64, p, p, p, p, p, p, p, p, p,
                                             C.POINTER(Params), p, p, i64, i64, p, p]
        _lib = L
    return _lib


def _ptr(a):
    return None if a is None else a.ctypes.data_as(C.c_void_p)


def _c(a, dt):
    return np.ascontiguousarray(a, dtype=dt)


def boundary(tri, nverts):
    """Surface.cpp:104-122 -> (on_boundary uint8[V], number of boundary points)."""
    tri = _c(tri, np.uint32)
    ob = np.zeros(nverts, dtype=np.uint8)
    nb = lib().fo_boundary(nverts, tri.shape[0], _ptr(tri), _ptr(ob))
    return ob, int(nb)


def idx_map(on_boundary, bc):
    """FEMContext.cpp:224-240 -> (idx_map int32[V], num_unknowns)."""
    ob = _c(on_boundary, np.uint8)
    im = np.zeros(ob.shape[0], dtype=np.int32)
    n = lib().fo_idx_map(ob.shape[0], _ptr(ob), int(bc), _ptr(im))
    return im, int(n)


def pattern(tri, on_boundary, idx, bc):
    """Eigen-compressed pattern of the triplets (FEMContext.cpp:97-112)."""
    tri = _c(tri, np.uint32)
    ob = _c(on_boundary, np.uint8)
    idx = _c(idx, np.int32)
    L = lib()
    h = L.fo_pattern_build(ob.shape[0], tri.shape[0], _ptr(tri), _ptr(ob), _ptr(idx), int(bc))
    try:
        n = L.fo_pattern_rows(h)
        nnz = L.fo_pattern_nnz(h)
        rp = np.zeros(n + 1, dtype=np.int32)
        col = np.zeros(nnz, dtype=np.int32)
        slot = np.zeros(9 * tri.shape[0], dtype=np.int32)
        aslot = np.zeros(9 * tri.shape[0], dtype=np.int32)
        L.fo_pattern_copy(h, _ptr(rp), _ptr(col), _ptr(slot), _ptr(aslot))
    finally:
        L.fo_pattern_free(h)
    return rp, col, slot, aslot


def _suffix(dtype):
    return "f64" if np.dtype(dtype) == np.float64 else "f32"


def element_matrices(xyz, tri, velocity=(1.0, 0.0, 0.0), elem_vel=None, dtype=np.float64):
    """Local K, M, Adv blocks [9T] of FEMContext.cpp:70-202."""
    xyz = _c(xyz, np.float32)
    tri = _c(tri, np.uint32)
    T = tri.shape[0]
    vel = _c(velocity, np.float32)
    ev = None if elem_vel is None else _c(elem_vel, np.float32)
    K = np.zeros(9 * T, dtype=dtype)
    M = np.zeros(9 * T, dtype=dtype)
    A = np.zeros(9 * T, dtype=dtype)
    getattr(lib(), f"fo_element_matrices_{_suffix(dtype)}")(
        T, _ptr(xyz), _ptr(tri), 0 if ev is None else 1, _ptr(vel), _ptr(ev), _ptr(K), _ptr(M), _ptr(A))
    return K, M, A


def ordered_sum(slot, loc, nnz, scale=None):
    """Duplicate summation of setFromTriplets, in triplet order."""
    dtype = loc.dtype
    out = np.zeros(nnz, dtype=dtype)
    sc = None if scale is None else _c(scale, dtype)
    slot = _c(slot, np.int32)
    getattr(lib(), f"fo_sum_{_suffix(dtype)}")(slot.shape[0] // 9, _ptr(slot), _ptr(loc), _ptr(sc), nnz, _ptr(out))
    return out


class System:
    """Assembled system of one mesh: the FEMContext state of the reference.

    Holds on_boundary, idx_map, the CSR pattern (identical index arrays to
    Eigen's compressed column-major storage, since the pattern is symmetric)
    and K, M, Adv on it.  `adv_present` marks the entries that exist in the
    reference's own advection matrix (its filter ignores the BC).
    """

    def __init__(self, xyz, tri, bc=NEUMANN, dtype=np.float64, velocity=(1.0, 0.0, 0.0),
                 elem_vel=None, diffusivity=None, on_boundary=None):
        self.xyz = _c(xyz, np.float32)
        self.tri = _c(tri, np.uint32)
        self.V = self.xyz.shape[0]
        self.T = self.tri.shape[0]
        self.bc = bc
        self.dtype = np.dtype(dtype)
        if on_boundary is None:
            self.on_boundary, self.num_boundary = boundary(self.tri, self.V)
        else:
            self.on_boundary = _c(on_boundary, np.uint8)
            self.num_boundary = int(self.on_boundary.sum())
        self.idx, self.N = idx_map(self.on_boundary, bc)
        self.row_ptr, self.col, self.slot, self.adv_slot = pattern(self.tri, self.on_boundary, self.idx, bc)
        self.nnz = self.col.shape[0]
        self.Kloc, self.Mloc, self.Aloc = element_matrices(self.xyz, self.tri, velocity, elem_vel, dtype)
        self.diffusivity = None if diffusivity is None else _c(diffusivity, dtype)
        self.K = ordered_sum(self.slot, self.Kloc, self.nnz, self.diffusivity)
        self.M = ordered_sum(self.slot, self.Mloc, self.nnz)
        self.Adv = ordered_sum(self.adv_slot, self.Aloc, self.nnz)
        present = np.zeros(self.nnz, dtype=np.uint8)
        s = self.adv_slot[self.adv_slot >= 0]
        present[s] = 1
        self.adv_present = present

    @property
    def max_row_nonzeros(self):
        """FEMContext.cpp:207-219."""
        return int(np.max(np.diff(self.row_ptr))) if self.N else 0

    def scipy(self, which):
        import scipy.sparse as sp
        val = {"K": self.K, "M": self.M, "Adv": self.Adv}[which]
        return sp.csr_matrix((val, self.col, self.row_ptr), shape=(self.N, self.N))

    def gather(self, values):
        """get_surface_value_vector (CPUSolver.cpp:13-21)."""
        out = np.zeros(self.N, dtype=self.dtype)
        m = self.idx >= 0
        out[self.idx[m]] = np.asarray(values)[m]
        return out

    def scatter(self, vec):
        """map_vector_to_surface (CPUSolver.cpp:28-37): Dirichlet points read 0."""
        out = np.zeros(self.V, dtype=self.dtype)
        m = self.idx >= 0
        out[m] = np.asarray(vec)[self.idx[m]]
        return out

    def step(self, params: Params, u, v, a=None, nsteps=1, prev=None):
        """advance_time x nsteps on unknown-indexed fields (copies returned).
        prev: (u, v) one step before u, v, for the first step's extrapolated
        start (warm_start 2)."""
        u = _c(u, self.dtype).copy()
        v = _c(v, self.dtype).copy()
        a = np.zeros(self.N, dtype=self.dtype) if a is None else _c(a, self.dtype).copy()
        it = C.c_int64(0)
        pu = pv = None
        if prev is not None:
            pu, pv = _c(prev[0], self.dtype), _c(prev[1], self.dtype)
        params.prev_u = None if pu is None else pu.ctypes.data
        params.prev_v = None if pv is None else pv.ctypes.data
        try:
            flags = getattr(lib(), f"fo_step_{_suffix(self.dtype)}")(
                self.N, _ptr(self.row_ptr), _ptr(self.col), _ptr(self.M), _ptr(self.K), _ptr(self.Adv),
                C.byref(params), _ptr(u), _ptr(v), _ptr(a), int(nsteps), C.byref(it))
        finally:
            params.prev_u = params.prev_v = None
        return u, v, a, int(it.value), int(flags)

    def newmark_init(self, params: Params, u):
        a = np.zeros(self.N, dtype=self.dtype)
        getattr(lib(), f"fo_newmark_init_{_suffix(self.dtype)}")(
            self.N, _ptr(self.row_ptr), _ptr(self.col), _ptr(self.M), _ptr(self.K), C.byref(params),
            _ptr(_c(u, self.dtype)), _ptr(a))
        return a

    def pcg(self, val, b, x0=None, tol=1e-12, max_iter=0, nthreads=1):
        b = _c(b, self.dtype)
        x = np.zeros(self.N, dtype=self.dtype) if x0 is None else _c(x0, self.dtype).copy()
        rr = C.c_double(0)
        it = getattr(lib(), f"fo_pcg_{_suffix(self.dtype)}")(
            self.N, _ptr(self.row_ptr), _ptr(self.col), _ptr(_c(val, self.dtype)), _ptr(b), _ptr(x),
            float(tol), int(max_iter), 1 if x0 is None else 0, int(nthreads), C.byref(rr))
        return x, int(it), rr.value

    def adjoint_gray_scott(self, params: Params, u0, v0, target_u, target_v, nsteps, ckpt):
        """FP64 adjoint of the mass-weighted Gray-Scott loss -> (J, dJ/du0, dJ/dv0, [dF, dk, dDu, dDv])."""
        u0 = _c(u0, np.float64)
        v0 = _c(v0, np.float64)
        tu = None if target_u is None else _c(target_u, np.float64)
        tv = None if target_v is None else _c(target_v, np.float64)
        gu = np.zeros(self.N)
        gv = np.zeros(self.N)
        gp = np.zeros(4)
        J = lib().fo_adjoint_gray_scott_f64(self.N, _ptr(self.row_ptr), _ptr(self.col), _ptr(self.M), _ptr(self.K),
                                            C.byref(params), _ptr(u0), _ptr(v0), _ptr(tu), _ptr(tv), int(nsteps),
                                            int(ckpt), _ptr(gu), _ptr(gv), _ptr(gp))
        return J, gu, gv, gp

    def adjoint_advdiff(self, params: Params, D, u0, target, nsteps, ckpt):
        """FP64 adjoint of the explicit advection-diffusion step -> (J, dJ/du0, dJ/dD)."""
        assert self.dtype == np.float64
        D = _c(D, np.float64)
        gu = np.zeros(self.N)
        gD = np.zeros(self.T)
        J = lib().fo_adjoint_advdiff_f64(
            self.N, self.T, _ptr(self.row_ptr), _ptr(self.col), _ptr(self.slot), _ptr(self.M),
            _ptr(self.Adv), _ptr(self.Kloc), _ptr(D), _ptr(self.idx), _ptr(self.tri), C.byref(params),
            _ptr(_c(u0, np.float64)), _ptr(_c(target, np.float64)), int(nsteps), int(ckpt),
            _ptr(gu), _ptr(gD))
        return J, gu, gD


def params(equation, dt, **kw) -> Params:
    """fo_params with defaults: FP64 oracle tolerance, warm start, 1 thread."""
    p = Params()
    p.equation = equation
    p.dt = dt
    p.kappa = kw.get("kappa", 0.0)
    p.Du = kw.get("Du", 0.0)
    p.Dv = kw.get("Dv", 0.0)
    p.F = kw.get("F", 0.0)
    p.k = kw.get("k", 0.0)
    p.reaction_mode = kw.get("reaction_mode", 1)
    p.wave_scheme = kw.get("wave_scheme", 0)
    p.beta = kw.get("beta", 0.25)
    p.gamma = kw.get("gamma", 0.5)
    p.adv_scheme = kw.get("adv_scheme", 0)
    p.adv_sign = kw.get("adv_sign", 1.0)
    p.k_scaled = kw.get("k_scaled", 0)
    p.tol = kw.get("tol", 1e-13)
    p.max_iter = kw.get("max_iter", 0)
    p.warm_start = kw.get("warm_start", 1)
    p.nthreads = kw.get("nthreads", 1)
    return p


def smooth_normals(xyz, tri, normals, values, extrusion):
    """Extruded smooth normals (smooth_normals.glsl), summed in triangle order -> float32[V, 3]."""
    xyz = _c(xyz, np.float32)
    tri = _c(tri, np.uint32)
    nrm = _c(normals, np.float32)
    val = _c(values, np.float32)
    out = np.zeros((xyz.shape[0], 3), dtype=np.float32)
    lib().fo_smooth_normals_f32(xyz.shape[0], tri.shape[0], _ptr(xyz), _ptr(tri), _ptr(nrm), _ptr(val),
                                float(extrusion), _ptr(out))
    return out


def ply_clip(xyz, tri, normals, values, extrusion, threshold, mesh_type):
    """Geometry of Surface::export_to_ply -> (positions float32[n, 3], values float32[n], triangles uint32[m, 3])."""
    xyz = _c(xyz, np.float32)
    tri = _c(tri, np.uint32)
    nrm = _c(normals, np.float32)
    val = _c(values, np.float32)
    T = tri.shape[0]
    cap_v, cap_t = 6 * T + 1, 4 * T + 1
    pos = np.zeros((cap_v, 3), dtype=np.float32)
    pv = np.zeros(cap_v, dtype=np.float32)
    tout = np.zeros((cap_t, 3), dtype=np.uint32)
    nt = C.c_int64(0)
    n = lib().fo_ply_clip(xyz.shape[0], T, _ptr(xyz), _ptr(tri), _ptr(nrm), _ptr(val), float(extrusion),
                          float(threshold), int(mesh_type), _ptr(pos), _ptr(pv), cap_v, _ptr(tout), cap_t,
                          C.byref(nt))
    return pos[:n].copy(), pv[:n].copy(), tout[:nt.value].copy()
