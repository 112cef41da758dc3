"""ctypes front-end of the CPU oracle (oracle.cpp).

TEST INFRASTRUCTURE ONLY: imported by tests/, by __graft_entry__.smoke() and
by bench.py's CPU-baseline legs, always as the checker.  The product library
never imports this module.
"""
import ctypes as C
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "_build", "liboracle.so")


def build(force=False):
    src = os.path.join(HERE, "oracle.cpp")
    if force or not os.path.exists(LIB_PATH) or os.path.getmtime(LIB_PATH) < os.path.getmtime(src):
        subprocess.check_call(["make", "-s", "-C", HERE, "_build/liboracle.so"])
    return LIB_PATH


class MeshDesc(C.Structure):
    _fields_ = [("nx", C.c_int), ("ny", C.c_int), ("nz", C.c_int), ("split", C.c_int),
                ("lo", C.c_double), ("hi", C.c_double), ("mapping", C.c_int),
                ("jitter", C.c_double), ("seed", C.c_uint64), ("periodic", C.c_int)]


class StepCfg(C.Structure):
    _fields_ = [("deposit_mode", C.c_int), ("solver", C.c_int), ("tol", C.c_double),
                ("max_iter", C.c_int), ("warm_start", C.c_int), ("gather_mode", C.c_int),
                ("kill", C.c_int), ("max_cross", C.c_int), ("compact_mode", C.c_int),
                ("nthreads", C.c_int)]


class StepStats(C.Structure):
    _fields_ = [("ke", C.c_double), ("n_alive", C.c_int64), ("n_killed", C.c_int64),
                ("n_cross", C.c_int64), ("n_walk_limit", C.c_int64), ("solver_iters", C.c_int),
                ("solver_resid", C.c_double)]


_lib = None


def lib():
    global _lib
    if _lib is None:
        build()
        L = C.CDLL(LIB_PATH)
        P = C.c_void_p
        I64, I32, D = C.c_int64, C.c_int, C.c_double
        L.orc_mesh_create.restype = P
        L.orc_mesh_create.argtypes = [C.POINTER(MeshDesc), C.c_char_p, I32]
        L.orc_mesh_destroy.argtypes = [P]
        L.orc_mesh_sizes.argtypes = [P] + [C.POINTER(I64)] * 5
        L.orc_mesh_export.argtypes = [P] * 9
        L.orc_mesh_export_periodic.argtypes = [P] * 3
        L.orc_csr_rows.restype = I64
        L.orc_csr_rows.argtypes = [P]
        L.orc_assemble.restype = I64
        L.orc_assemble.argtypes = [P, I32]
        L.orc_csr_export.argtypes = [P, P, P, P]
        L.orc_spmv.argtypes = [P, P, P, I32]
        L.orc_background.argtypes = [P, D, P]
        L.orc_deposit.argtypes = [P, I32, I64, P, P, P, P, P, P, P, I32]
        L.orc_deposit_fixed.argtypes = [P, I64, P, P, P, P]
        L.orc_bicgstab.restype = I32
        L.orc_bicgstab.argtypes = [P, P, P, D, I32, C.POINTER(D), I32]
        L.orc_cg.restype = I32
        L.orc_cg.argtypes = [P, P, P, D, I32, C.POINTER(D), I32]
        L.orc_efield_tet.argtypes = [P, P, P, I32]
        L.orc_gather.argtypes = [P, I32, I64, P, P, P, P, P, I32]
        L.orc_push.argtypes = [P, I64, P, P, P, P, P, P, D, I32]
        L.orc_walk.restype = I64
        L.orc_walk.argtypes = [P, I64, P, P, P, P, P, D, I32, I32, C.POINTER(I64), C.POINTER(I64), I32]
        L.orc_compact.restype = I64
        L.orc_compact.argtypes = [I32, I64, P, P, P, P, P, P, P]
        L.orc_kinetic.restype = D
        L.orc_sort_by_cell.restype = I64
        L.orc_sort_by_cell.argtypes = [I64, P, I64, P, P]
        L.orc_kinetic.argtypes = [I64, P, P, P, P, I32]
        L.orc_fill_ref.restype = I64
        L.orc_fill_ref.argtypes = [P, I32, I32, D, P, D, D, I64, P, P, P, P, P, P]
        L.orc_fill_uniform.argtypes = [P, I64, C.c_uint64, I32, D, P, D, P, P, P, P, P, P, I32]
        L.orc_ref_lcg.argtypes = [C.c_uint64, I32, P, P]
        L.orc_mix64.restype = C.c_uint64
        L.orc_mix64.argtypes = [C.c_uint64]
        L.orc_draw.restype = C.c_uint64
        L.orc_draw.argtypes = [C.c_uint64, C.c_uint64]
        L.orc_step.restype = I32
        L.orc_step.argtypes = [P, C.POINTER(StepCfg), D, C.POINTER(I64)] + [P] * 14 + [C.POINTER(StepStats)]
        _lib = L
    return _lib


def ptr(a):
    return None if a is None else a.ctypes.data_as(C.c_void_p)


class Mesh:
    """Oracle mesh (mesh.cpp:78-714 restated)."""

    def __init__(self, n, split=6, lo=0.0, hi=1.0, mapping=0, jitter=0.0, seed=0, periodic=0):
        nx, ny, nz = (n, n, n) if np.isscalar(n) else n
        self.desc = MeshDesc(nx, ny, nz, split, lo, hi, mapping, jitter, seed, int(periodic))
        self.periodic = int(periodic)
        err = C.create_string_buffer(256)
        self.h = lib().orc_mesh_create(C.byref(self.desc), err, 256)
        if not self.h:
            raise ValueError(err.value.decode())
        v = [C.c_int64() for _ in range(5)]
        lib().orc_mesh_sizes(self.h, *[C.byref(x) for x in v])
        self.T, self.N, self.n_faces, self.n_bfaces, self.n_bnodes = [x.value for x in v]
        T, N = self.T, self.N
        self.nodes = np.zeros((N, 3))
        self.tets = np.zeros((T, 4), np.int32)
        self.nbrs = np.zeros((T, 4), np.int32)
        self.jinv = np.zeros((T, 9))
        self.detj = np.zeros(T)
        self.normals = np.zeros((T, 12))
        self.grad = np.zeros((T, 12))
        self.boundary = np.zeros(N, np.uint8)
        lib().orc_mesh_export(self.h, *[ptr(a) for a in (self.nodes, self.tets, self.nbrs, self.jinv, self.detj,
                                                          self.normals, self.grad, self.boundary)])
        self.face_periodic = np.zeros((T, 4), np.int8)
        self.node_pairs = np.zeros(N, np.int32)
        lib().orc_mesh_export_periodic(self.h, ptr(self.face_periodic), ptr(self.node_pairs))
        self.csr = None

    def __del__(self):
        if getattr(self, "h", None) and _lib is not None:
            _lib.orc_mesh_destroy(self.h)
            self.h = None

    def assemble(self, mode=1):
        nnz = lib().orc_assemble(self.h, mode)
        rp = np.zeros(lib().orc_csr_rows(self.h) + 1, np.int32)
        col = np.zeros(nnz, np.int32)
        val = np.zeros(nnz)
        lib().orc_csr_export(self.h, ptr(rp), ptr(col), ptr(val))
        self.csr = (rp, col, val)
        self.csr_mode = mode
        return self.csr

    def spmv(self, x, nthreads=1):
        y = np.zeros(self.N)
        lib().orc_spmv(self.h, ptr(np.ascontiguousarray(x, np.float64)), ptr(y), nthreads)
        return y

    def background(self, rho_bg):
        bg = np.zeros(self.N)
        lib().orc_background(self.h, rho_bg, ptr(bg))
        return bg

    def efield_tet(self, phi, nthreads=1):
        E = np.zeros((self.T, 3))
        lib().orc_efield_tet(self.h, ptr(np.ascontiguousarray(phi, np.float64)), ptr(E), nthreads)
        return E


class Particles:
    """Plain FP64 particle state in SoA numpy arrays (row p = particle p)."""

    def __init__(self, cap):
        self.n = 0
        self.cell = np.full(cap, -1, np.int32)
        self.x = np.zeros((cap, 3))
        self.xref = np.zeros((cap, 3))
        self.v = np.zeros((cap, 3))
        self.vref = np.zeros((cap, 3))
        self.w = np.zeros(cap)
        self.sp = np.zeros(cap, np.int32)
        self.id = np.arange(cap, dtype=np.int64)

    @property
    def cap(self):
        return self.cell.shape[0]

    def view(self, name):
        return getattr(self, name)[: self.n]

    def fill_ref(self, mesh, nppe, type_, density, vel=(0, 0, 0), temp=1.0, mass=1.0):
        k0 = self.n
        vel = np.asarray(vel, np.float64)
        cnt = lib().orc_fill_ref(mesh.h, nppe, type_, density, ptr(vel), temp, mass, self.cap - k0,
                                 ptr(self.cell[k0:]), ptr(self.x[k0:]), ptr(self.xref[k0:]), ptr(self.v[k0:]),
                                 ptr(self.w[k0:]), ptr(self.sp[k0:]))
        if cnt < 0:
            raise ValueError("capacity")
        self.n += cnt
        return cnt

    def fill_uniform(self, mesh, n, seed, type_, weight, drift=(0, 0, 0), vth=0.05, nthreads=0):
        k0 = self.n
        if k0 + n > self.cap:
            raise ValueError("capacity")
        drift = np.asarray(drift, np.float64)
        lib().orc_fill_uniform(mesh.h, n, seed, type_, weight, ptr(drift), vth, ptr(self.cell[k0:]),
                               ptr(self.x[k0:]), ptr(self.xref[k0:]), ptr(self.v[k0:]), ptr(self.w[k0:]),
                               ptr(self.sp[k0:]), nthreads)
        self.n += n
        return n


def ref_lcg(seed, n):
    r = np.zeros(n, np.uint64)
    d = np.zeros(n)
    lib().orc_ref_lcg(seed, n, ptr(r), ptr(d))
    return r, d


def deposit(mesh, parts, mode, q_of_species, bg=None, nthreads=1):
    rhs = np.zeros(mesh.N)
    q = np.zeros(16)
    q[: len(q_of_species)] = q_of_species
    lib().orc_deposit(mesh.h, mode, parts.n, ptr(parts.cell), ptr(parts.xref), ptr(parts.w), ptr(parts.sp), ptr(q),
                      ptr(bg), ptr(rhs), nthreads)
    return rhs


def deposit_fixed(mesh, cellsp, b, qfix_of_species):
    acc = np.zeros(mesh.N, np.int64)
    q = np.zeros(256, np.int64)
    q[: len(qfix_of_species)] = qfix_of_species
    lib().orc_deposit_fixed(mesh.h, len(cellsp), ptr(np.ascontiguousarray(cellsp, np.uint32)),
                            ptr(np.ascontiguousarray(b, np.float32)), ptr(q), ptr(acc))
    return acc


def bicgstab(mesh, rhs, tol=1e-6, max_iter=1000, nthreads=1):
    x = np.zeros(mesh.N)
    r = C.c_double()
    it = lib().orc_bicgstab(mesh.h, ptr(np.ascontiguousarray(rhs)), ptr(x), tol, max_iter, C.byref(r), nthreads)
    return x, it, r.value


def cg(mesh, rhs, x0=None, tol=1e-10, max_iter=1000, nthreads=1):
    x = np.zeros(mesh.N) if x0 is None else np.array(x0, np.float64)
    r = C.c_double()
    it = lib().orc_cg(mesh.h, ptr(np.ascontiguousarray(rhs)), ptr(x), tol, max_iter, C.byref(r), nthreads)
    return x, it, r.value


def gather(mesh, parts, mode, phi, E_tet=None, nthreads=1):
    E = np.zeros((parts.n, 3))
    lib().orc_gather(mesh.h, mode, parts.n, ptr(parts.cell), ptr(parts.xref), ptr(np.ascontiguousarray(phi)),
                     ptr(E_tet), ptr(E), nthreads)
    return E


def push(mesh, parts, E, qm_of_species, dt, nthreads=1):
    qm = np.zeros(16)
    qm[: len(qm_of_species)] = qm_of_species
    lib().orc_push(mesh.h, parts.n, ptr(parts.cell), ptr(np.ascontiguousarray(E)), ptr(parts.v), ptr(parts.vref),
                   ptr(parts.sp), ptr(qm), dt, nthreads)


def walk(mesh, parts, dt, kill=1, max_cross=1000, nthreads=1):
    nk, nc = C.c_int64(), C.c_int64()
    lim = lib().orc_walk(mesh.h, parts.n, ptr(parts.cell), ptr(parts.x), ptr(parts.xref), ptr(parts.v),
                         ptr(parts.vref), dt, kill, max_cross, C.byref(nk), C.byref(nc), nthreads)
    return dict(limit=lim, killed=nk.value, cross=nc.value)


def compact(parts, mode=1):
    parts.n = lib().orc_compact(mode, parts.n, ptr(parts.cell), ptr(parts.x), ptr(parts.xref), ptr(parts.v),
                                ptr(parts.w), ptr(parts.sp), ptr(parts.id))
    return parts.n


def sort_by_cell(cell, T):
    """Stable sort by element (ParticleList::sort, particle_list.cpp:90-146):
    (perm, start) with perm[k] the input index of sorted position k (dead
    entries, cell < 0, dropped) and start[e] the first position of element e."""
    cell = np.ascontiguousarray(cell, np.int32)
    perm = np.zeros(len(cell), np.int64)
    start = np.zeros(T + 1, np.int64)
    m = lib().orc_sort_by_cell(len(cell), ptr(cell), T, ptr(perm), ptr(start))
    return perm[:m], start


def kinetic(parts, m_of_species):
    m = np.zeros(16)
    m[: len(m_of_species)] = m_of_species
    return lib().orc_kinetic(parts.n, ptr(parts.v), ptr(parts.w), ptr(parts.sp), ptr(m), 1)


def step(mesh, parts, cfg, dt, q_of_species, m_of_species, bg, phi, scratch=None):
    q = np.zeros(16)
    q[: len(q_of_species)] = q_of_species
    m = np.zeros(16)
    m[: len(m_of_species)] = m_of_species
    rhs = np.zeros(mesh.N)
    E = scratch if scratch is not None else np.zeros((parts.cap, 3))
    n = C.c_int64(parts.n)
    st = StepStats()
    rc = lib().orc_step(mesh.h, C.byref(cfg), dt, C.byref(n), ptr(parts.cell), ptr(parts.x), ptr(parts.xref),
                        ptr(parts.v), ptr(parts.vref), ptr(parts.w), ptr(parts.sp), ptr(parts.id), ptr(q), ptr(m),
                        ptr(bg), ptr(phi), ptr(rhs), ptr(E), C.byref(st))
    parts.n = n.value
    return rc, st, rhs
