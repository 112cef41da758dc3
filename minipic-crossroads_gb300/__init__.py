"""Python front-end of the GB300 PIC library (ctypes over include/minipic_gb300.h).

The library itself is C++/CUDA (csrc/); this module only loads
_build/libminipic_gb300.so and wraps the C ABI for tests and benchmarks.  It
has no CPU fallback: if the shared library or a CUDA device is missing, the
calls raise.
"""
import ctypes as C
import os

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))

OK = 0
ERR_ARG, ERR_CUDA, ERR_CAPACITY, ERR_WALK_LIMIT, ERR_NAN, ERR_NOT_CONVERGED, ERR_STATE, ERR_MESH, ERR_TIMEOUT = \
    -1, -2, -3, -4, -5, -6, -7, -8, -9
PLAIN, MIXED = 0, 1
DEPOSIT_REF_QUARTER, DEPOSIT_LINEAR = 0, 1
SOLVER_BICGSTAB, SOLVER_CG, SOLVER_CG_MG = 0, 1, 2
SPLIT_REF5, SPLIT_KUHN6 = 5, 6
MAP_NONE, MAP_JITTER = 0, 4
FIELD_RHS, FIELD_PHI, FIELD_E_TET, FIELD_BACKGROUND = 0, 1, 2, 3
DEAD = 0xFFFFFFFF

# every symbol include/minipic_gb300.h declares
EXPORTS = [
    "mpg_version", "mpg_device_count", "mpg_ctx_create", "mpg_ctx_destroy", "mpg_last_error", "mpg_set_timing",
    "mpg_timer",
    "mpg_mesh_build", "mpg_mesh_sizes", "mpg_mesh_download", "mpg_mesh_periodic_download", "mpg_species_set",
    "mpg_configure", "mpg_csr_sizes",
    "mpg_csr_download", "mpg_particles_reserve", "mpg_fill_ref", "mpg_fill_uniform", "mpg_particles_upload",
    "mpg_particles_download", "mpg_particles_count", "mpg_mixed_download", "mpg_mixed_upload",
    "mpg_charge_download", "mpg_weight_charge", "mpg_solve", "mpg_weight_efield", "mpg_move", "mpg_step",
    "mpg_sort", "mpg_cell_starts", "mpg_set_barrier_test", "mpg_get_field", "mpg_set_field", "mpg_cg_csr", "mpg_cg_csr_noalloc", "mpg_mg_hierarchy",
    "mpg_batch_create", "mpg_batch_destroy", "mpg_batch_last_error", "mpg_batch_set_tuning", "mpg_batch_set_fused",
    "mpg_batch_admit",
    "mpg_batch_prepare", "mpg_batch_admit_prepared", "mpg_run_prep_destroy",
    "mpg_batch_step", "mpg_batch_run_info", "mpg_batch_run_phi", "mpg_batch_run_particles", "mpg_batch_retire",
]
NOALLOC_MAX_N = 131072


class MeshDesc(C.Structure):
    _fields_ = [("nx", C.c_int), ("ny", C.c_int), ("nz", C.c_int), ("split", C.c_int), ("lo", C.c_double),
                ("hi", C.c_double), ("mapping", C.c_int), ("jitter", C.c_double), ("seed", C.c_uint64),
                ("periodic", C.c_int)]


class Config(C.Structure):
    _fields_ = [("precision", C.c_int), ("deposit", C.c_int), ("solver", C.c_int), ("tol", C.c_double),
                ("max_iter", C.c_int), ("warm_start", C.c_int), ("kill_on_wall", C.c_int),
                ("max_crossings", C.c_int), ("sort_interval", C.c_int), ("rho_background", C.c_double),
                ("track_ids", C.c_int)]


class StepStats(C.Structure):
    _fields_ = [("ke", C.c_double), ("n_alive", C.c_int64), ("n_killed", C.c_int64), ("n_crossings", C.c_int64),
                ("n_walk_limit", C.c_int64), ("solver_iters", C.c_int), ("solver_resid", C.c_double),
                ("status", C.c_int), ("steps", C.c_int), ("ms_deposit", C.c_double), ("ms_solve", C.c_double),
                ("ms_efield", C.c_double), ("ms_move", C.c_double), ("ms_sort", C.c_double),
                ("n_launches", C.c_int64)]

    def as_dict(self):
        return {k: getattr(self, k) for k, _ in self._fields_}


class RunDesc(C.Structure):
    _fields_ = [("n_side", C.c_int), ("n_particles", C.c_int64), ("seed", C.c_uint64), ("q", C.c_double),
                ("m", C.c_double), ("weight", C.c_double), ("vth", C.c_double), ("drift", C.c_double * 3),
                ("rho_background", C.c_double), ("dt", C.c_double), ("tol", C.c_double), ("max_iter", C.c_int),
                ("steps", C.c_int), ("jitter", C.c_double), ("mesh_seed", C.c_uint64)]


class RunInfo(C.Structure):
    _fields_ = [("active", C.c_int), ("finished", C.c_int), ("steps_done", C.c_int), ("n_alive", C.c_int64),
                ("ke", C.c_double), ("solver_iters", C.c_int), ("solver_resid", C.c_double), ("status", C.c_int),
                ("bytes", C.c_int64)]


class BatchStats(C.Structure):
    _fields_ = [("active_runs", C.c_int), ("particle_steps", C.c_int64), ("ms", C.c_double),
                ("ms_last_step", C.c_double), ("n_launches", C.c_int64), ("graph", C.c_int), ("status", C.c_int)]


def lib_path():
    return os.path.join(HERE, "_build", "libminipic_gb300.so")


def build(force=False):
    import importlib.util
    spec = importlib.util.spec_from_file_location("_mpg_build", os.path.join(HERE, "build.py"))
    mod = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(mod)
    return mod.build(force=force)


_lib = None


def load():
    """Load the shared library (raises if it is missing: there is no fallback)."""
    global _lib
    if _lib is not None:
        return _lib
    path = lib_path()
    if not os.path.exists(path):
        raise RuntimeError(f"{path} is missing: build the CUDA library first (__graft_entry__.build())")
    L = C.CDLL(path)
    P, I, I64, D, U64 = C.c_void_p, C.c_int, C.c_int64, C.c_double, C.c_uint64
    sig = {
        "mpg_version": ([], I),
        "mpg_device_count": ([C.POINTER(I)], I),
        "mpg_ctx_create": ([I, C.POINTER(P)], I),
        "mpg_ctx_destroy": ([P], I),
        "mpg_last_error": ([P, C.c_char_p, I], I),
        "mpg_set_timing": ([P, I], I),
        "mpg_timer": ([P, I, C.POINTER(D)], I),
        "mpg_mesh_build": ([P, C.POINTER(MeshDesc)], I),
        "mpg_mesh_sizes": ([P, C.POINTER(I64), C.POINTER(I64), C.POINTER(I64)], I),
        "mpg_mesh_download": ([P] * 8, I),
        "mpg_mesh_periodic_download": ([P] * 3, I),
        "mpg_species_set": ([P, I, D, D], I),
        "mpg_configure": ([P, C.POINTER(Config)], I),
        "mpg_csr_sizes": ([P, C.POINTER(I64), C.POINTER(I64)], I),
        "mpg_csr_download": ([P, P, P, P], I),
        "mpg_particles_reserve": ([P, I64], I),
        "mpg_fill_ref": ([P, I, I, D, P, D], I),
        "mpg_fill_uniform": ([P, I64, U64, I, D, P, D], I),
        "mpg_particles_upload": ([P, I64] + [P] * 7, I),
        "mpg_particles_download": ([P, I64, C.POINTER(I64)] + [P] * 7, I),
        "mpg_particles_count": ([P, C.POINTER(I64)], I),
        "mpg_mixed_download": ([P, I64, C.POINTER(I64), P, P, P], I),
        "mpg_mixed_upload": ([P, I64, P, P, P], I),
        "mpg_charge_download": ([P, P, C.POINTER(D), P], I),
        "mpg_weight_charge": ([P], I),
        "mpg_solve": ([P, C.POINTER(I), C.POINTER(D)], I),
        "mpg_weight_efield": ([P], I),
        "mpg_move": ([P, D, C.POINTER(StepStats)], I),
        "mpg_step": ([P, D, I, C.POINTER(StepStats)], I),
        "mpg_sort": ([P], I),
        "mpg_cell_starts": ([P, I64, P], I),
        "mpg_set_barrier_test": ([P, I, C.c_uint], I),
        "mpg_get_field": ([P, I, P], I),
        "mpg_set_field": ([P, I, P], I),
        "mpg_cg_csr": ([P, I64, P, P, P, P, P, D, I, C.POINTER(I), C.POINTER(D)], I),
        "mpg_cg_csr_noalloc": ([P, I64, P, P, P, P, P, D, I, C.POINTER(I), C.POINTER(D)], I),
        "mpg_mg_hierarchy": ([C.POINTER(MeshDesc), I64, I, C.POINTER(I), P, P, P, P], I),
        "mpg_batch_create": ([I, I64, I, I64, C.POINTER(P)], I),
        "mpg_batch_destroy": ([P], I),
        "mpg_batch_last_error": ([P, C.c_char_p, I], I),
        "mpg_batch_set_tuning": ([P, I, I], I),
        "mpg_batch_set_fused": ([P, I], I),
        "mpg_batch_admit": ([P, C.POINTER(RunDesc), C.POINTER(I)], I),
        "mpg_batch_prepare": ([C.POINTER(RunDesc), C.POINTER(P)], I),
        "mpg_batch_admit_prepared": ([P, P, C.POINTER(I)], I),
        "mpg_run_prep_destroy": ([P], I),
        "mpg_batch_step": ([P, I, C.POINTER(BatchStats)], I),
        "mpg_batch_run_info": ([P, I, C.POINTER(RunInfo)], I),
        "mpg_batch_run_phi": ([P, I, P], I),
        "mpg_batch_run_particles": ([P, I, I64, C.POINTER(I64), P, P, P], I),
        "mpg_batch_retire": ([P, I], I),
    }
    for name, (args, res) in sig.items():
        f = getattr(L, name)
        f.argtypes = args
        f.restype = res
    _lib = L
    return L


def ptr(a):
    return None if a is None else a.ctypes.data_as(C.c_void_p)


class MpgError(RuntimeError):
    def __init__(self, code, msg):
        super().__init__(f"[{code}] {msg}")
        self.code = code


def mg_hierarchy(n, split=SPLIT_KUHN6, lo=0.0, hi=1.0, mapping=MAP_NONE, jitter=0.0, seed=0, periodic=0,
                 dense_max=0, level=0):
    """Level `level` of the multigrid hierarchy MPG_SOLVER_CG_MG builds for a
    mesh, computed on the host only (no GPU): dict(nlev, extent, val [27, n]
    (levels >= 1), dinv [n], bnd [n])."""
    L = load()
    nx, ny, nz = (n, n, n) if np.isscalar(n) else n
    d = MeshDesc(nx, ny, nz, split, lo, hi, mapping, jitter, seed, int(periodic))
    nlev, ext = C.c_int(), (C.c_int * 3)()
    rc = L.mpg_mg_hierarchy(C.byref(d), dense_max, level, C.byref(nlev), ext, None, None, None)
    if rc != OK:
        raise MpgError(rc, "mpg_mg_hierarchy failed")
    m = ext[0] * ext[1] * ext[2]
    val = np.zeros((27, m), np.float32) if level > 0 else None
    dinv, bnd = np.zeros(m, np.float32), np.zeros(m, np.uint8)
    rc = L.mpg_mg_hierarchy(C.byref(d), dense_max, level, C.byref(nlev), ext, ptr(val), ptr(dinv), ptr(bnd))
    if rc != OK:
        raise MpgError(rc, "mpg_mg_hierarchy failed")
    return dict(nlev=nlev.value, extent=(ext[0], ext[1], ext[2]), val=val, dinv=dinv, bnd=bnd)


class Ctx:
    """One device-resident PIC run (DataWarehouse + Mesh + ParticleList + ES + PIC)."""

    def __init__(self, device=0):
        self.L = load()
        h = C.c_void_p()
        rc = self.L.mpg_ctx_create(device, C.byref(h))
        if rc != OK:
            buf = C.create_string_buffer(512)
            self.L.mpg_last_error(None, buf, 512)
            raise MpgError(rc, buf.value.decode())
        self.h = h
        self.T = self.N = 0

    def close(self):
        if getattr(self, "h", None):
            self.L.mpg_ctx_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()

    def _ck(self, rc, allow=()):
        if rc != OK and rc not in allow:
            buf = C.create_string_buffer(512)
            self.L.mpg_last_error(self.h, buf, 512)
            raise MpgError(rc, buf.value.decode())
        return rc

    def last_error(self):
        buf = C.create_string_buffer(512)
        self.L.mpg_last_error(self.h, buf, 512)
        return buf.value.decode()

    def set_timing(self, on=True):
        self._ck(self.L.mpg_set_timing(self.h, int(on)))

    def timer_start(self):
        self._ck(self.L.mpg_timer(self.h, 0, None))

    def timer_stop(self):
        ms = C.c_double()
        self._ck(self.L.mpg_timer(self.h, 1, C.byref(ms)))
        return ms.value

    def mesh(self, n, split=SPLIT_KUHN6, lo=0.0, hi=1.0, mapping=MAP_NONE, jitter=0.0, seed=0, periodic=0):
        nx, ny, nz = (n, n, n) if np.isscalar(n) else n
        d = MeshDesc(nx, ny, nz, split, lo, hi, mapping, jitter, seed, int(periodic))
        self._ck(self.L.mpg_mesh_build(self.h, C.byref(d)))
        T, N, nb = C.c_int64(), C.c_int64(), C.c_int64()
        self._ck(self.L.mpg_mesh_sizes(self.h, C.byref(T), C.byref(N), C.byref(nb)))
        self.T, self.N, self.n_bnodes = T.value, N.value, nb.value
        return self

    def mesh_arrays(self):
        T, N = self.T, self.N
        out = dict(nodes=np.zeros((N, 3)), tets=np.zeros((T, 4), np.int32), nbrs=np.zeros((T, 4), np.int32),
                   jinv=np.zeros((T, 9)), detj=np.zeros(T), normals=np.zeros((T, 12)),
                   boundary=np.zeros(N, np.uint8))
        self._ck(self.L.mpg_mesh_download(self.h, *[ptr(out[k]) for k in
                                                    ("nodes", "tets", "nbrs", "jinv", "detj", "normals",
                                                     "boundary")]))
        return out

    def periodic_arrays(self):
        """(face_periodic (T,4) int8, node_pairs (N,) int32) of a periodic mesh."""
        fp = np.zeros((self.T, 4), np.int8)
        pr = np.zeros(self.N, np.int32)
        self._ck(self.L.mpg_mesh_periodic_download(self.h, ptr(fp), ptr(pr)))
        return fp, pr

    def species(self, i, q, m):
        self._ck(self.L.mpg_species_set(self.h, i, q, m))

    def configure(self, precision=PLAIN, deposit=DEPOSIT_REF_QUARTER, solver=SOLVER_BICGSTAB, tol=1e-6,
                  max_iter=1000, warm_start=0, kill_on_wall=0, max_crossings=1000, sort_interval=0,
                  rho_background=0.0, track_ids=0):
        self.cfg = Config(precision, deposit, solver, tol, max_iter, warm_start, kill_on_wall, max_crossings,
                          sort_interval, rho_background, track_ids)
        self._ck(self.L.mpg_configure(self.h, C.byref(self.cfg)))
        return self

    def csr(self):
        rows, nnz = C.c_int64(), C.c_int64()
        self._ck(self.L.mpg_csr_sizes(self.h, C.byref(rows), C.byref(nnz)))
        rp = np.zeros(rows.value + 1, np.int32)
        col = np.zeros(nnz.value, np.int32)
        val = np.zeros(nnz.value)
        self._ck(self.L.mpg_csr_download(self.h, ptr(rp), ptr(col), ptr(val)))
        return rp, col, val

    def reserve(self, cap):
        self._ck(self.L.mpg_particles_reserve(self.h, int(cap)))

    def fill_ref(self, nppe, type_, density, vel=(0.0, 0.0, 0.0), temp=1.0):
        v = np.asarray(vel, np.float64)
        return self._ck(self.L.mpg_fill_ref(self.h, nppe, type_, density, ptr(v), temp), allow=(ERR_CAPACITY,))

    def fill_uniform(self, n, seed, type_, weight, drift=(0.0, 0.0, 0.0), vth=0.05):
        d = np.asarray(drift, np.float64)
        self._ck(self.L.mpg_fill_uniform(self.h, int(n), seed, type_, weight, ptr(d), vth))

    def upload(self, cell, x, xref, v, w=None, sp=None, ids=None):
        n = len(cell)
        arrs = [np.ascontiguousarray(cell, np.int32), None if x is None else np.ascontiguousarray(x, np.float64),
                np.ascontiguousarray(xref, np.float64), np.ascontiguousarray(v, np.float64),
                None if w is None else np.ascontiguousarray(w, np.float64),
                None if sp is None else np.ascontiguousarray(sp, np.int32),
                None if ids is None else np.ascontiguousarray(ids, np.int64)]
        self._ck(self.L.mpg_particles_upload(self.h, n, *[ptr(a) for a in arrs]))

    def count(self):
        n = C.c_int64()
        self._ck(self.L.mpg_particles_count(self.h, C.byref(n)))
        return n.value

    def download(self, cap=None):
        if cap is None:
            cap = self.slots()
        cap = max(int(cap), 1)
        out = dict(cell=np.zeros(cap, np.int32), x=np.zeros((cap, 3)), xref=np.zeros((cap, 3)),
                   v=np.zeros((cap, 3)), w=np.zeros(cap), sp=np.zeros(cap, np.int32), id=np.zeros(cap, np.int64))
        n = C.c_int64()
        self._ck(self.L.mpg_particles_download(self.h, cap, C.byref(n), *[ptr(out[k]) for k in
                                                                          ("cell", "x", "xref", "v", "w", "sp",
                                                                           "id")]))
        return {k: a[: n.value] for k, a in out.items()}

    def slots(self):
        # upper bound of particle slots (live + holes); download returns this many
        n = C.c_int64()
        cap = 1 << 31
        self._ck(self.L.mpg_particles_download(self.h, 0, C.byref(n), None, None, None, None, None, None, None),
                 allow=(ERR_CAPACITY,))
        del cap
        return n.value

    def mixed_download(self, out=None):
        """(cellsp, barycentrics, velocities) of the live slots; `out` = three
        caller arrays (uint32 [cap], float32 [cap, 3] x 2, e.g. pinned host
        memory) to download into instead of fresh ones."""
        if out is None:
            cap = max(self.slots(), 1)
            cs = np.zeros(cap, np.uint32)
            b = np.zeros((cap, 3), np.float32)
            v = np.zeros((cap, 3), np.float32)
        else:
            cs, b, v = out
            if cs.dtype != np.uint32 or b.dtype != np.float32 or v.dtype != np.float32 or b.shape[1:] != (3,) \
                    or v.shape[1:] != (3,) or not (len(cs) == len(b) == len(v)) or not all(
                        a.flags.c_contiguous for a in (cs, b, v)):
                raise ValueError("out must be contiguous uint32 [cap] and float32 [cap, 3] arrays")
            cap = len(cs)
        n = C.c_int64()
        self._ck(self.L.mpg_mixed_download(self.h, cap, C.byref(n), ptr(cs), ptr(b), ptr(v)))
        return cs[: n.value], b[: n.value], v[: n.value]

    def mixed_upload(self, cs, b, v):
        self._ck(self.L.mpg_mixed_upload(self.h, len(cs), ptr(np.ascontiguousarray(cs, np.uint32)),
                                         ptr(np.ascontiguousarray(b, np.float32)),
                                         ptr(np.ascontiguousarray(v, np.float32))))

    def charge(self):
        acc = np.zeros(self.N, np.int64)
        q = C.c_double()
        qfix = np.zeros(16, np.int64)
        self._ck(self.L.mpg_charge_download(self.h, ptr(acc), C.byref(q), ptr(qfix)))
        return acc, q.value, qfix

    def weight_charge(self):
        self._ck(self.L.mpg_weight_charge(self.h))

    def solve(self):
        it, res = C.c_int(), C.c_double()
        self._ck(self.L.mpg_solve(self.h, C.byref(it), C.byref(res)))
        return it.value, res.value

    def weight_efield(self):
        self._ck(self.L.mpg_weight_efield(self.h))

    def move(self, dt):
        st = StepStats()
        self._ck(self.L.mpg_move(self.h, dt, C.byref(st)))
        return st

    def step(self, dt, n=1, allow=()):
        st = StepStats()
        rc = self._ck(self.L.mpg_step(self.h, dt, n, C.byref(st)), allow=allow)
        st.rc = rc
        return st

    def sort(self):
        self._ck(self.L.mpg_sort(self.h))

    def barrier_test(self, skip_block=-1, poll_limit=0):
        """Make the field solves' grid barriers time out (block skip_block
        does not arrive; waits give up after poll_limit polls); -1 turns it off."""
        self._ck(self.L.mpg_set_barrier_test(self.h, int(skip_block), int(poll_limit)))

    def cell_starts(self):
        """start[e] = first list position of cell e after the last sort (T + 1 entries)."""
        a = np.zeros(self.T + 1, np.int64)
        self._ck(self.L.mpg_cell_starts(self.h, len(a), ptr(a)))
        return a

    def get_field(self, which):
        n = 3 * self.T if which == FIELD_E_TET else self.N
        a = np.zeros(n)
        self._ck(self.L.mpg_get_field(self.h, which, ptr(a)))
        return a.reshape(-1, 3) if which == FIELD_E_TET else a

    def set_field(self, which, a):
        self._ck(self.L.mpg_set_field(self.h, which, ptr(np.ascontiguousarray(a, np.float64))))


class Batch:
    """Many independent runs resident on one GPU, stepped together (mpg_batch_*)."""

    def __init__(self, device=0, budget_bytes=8 << 30, max_runs=256, particle_capacity=1 << 24):
        self.L = load()
        h = C.c_void_p()
        rc = self.L.mpg_batch_create(device, int(budget_bytes), int(max_runs), int(particle_capacity), C.byref(h))
        if rc != OK:
            raise MpgError(rc, "mpg_batch_create failed")
        self.h = h
        self.n_nodes = {}

    def close(self):
        if getattr(self, "h", None):
            self.L.mpg_batch_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def _ck(self, rc, allow=()):
        if rc != OK and rc not in allow:
            buf = C.create_string_buffer(512)
            self.L.mpg_batch_last_error(self.h, buf, 512)
            raise MpgError(rc, buf.value.decode())
        return rc

    def tuning(self, cg_threads=512, sort_interval=10, fused=None):
        self._ck(self.L.mpg_batch_set_tuning(self.h, cg_threads, sort_interval))
        if fused is not None:
            self._ck(self.L.mpg_batch_set_fused(self.h, int(fused)))

    @staticmethod
    def desc(n_side, n_particles, seed, q=-1.0, m=1.0, weight=None, vth=0.05, drift=(0.0, 0.0, 0.0),
             rho_background=None, dt=0.01, tol=1e-10, max_iter=5000, steps=100, jitter=0.0, mesh_seed=1):
        w = (1.0 / n_particles) if weight is None else weight
        rho = (-q * w * n_particles) if rho_background is None else rho_background
        return RunDesc(n_side, int(n_particles), seed, q, m, w, vth, (C.c_double * 3)(*drift), rho, dt, tol,
                       max_iter, steps, jitter, mesh_seed)

    def admit(self, n_side, n_particles, seed, allow=(), **kw):
        d = self.desc(n_side, n_particles, seed, **kw)
        slot = C.c_int(-1)
        rc = self._ck(self.L.mpg_batch_admit(self.h, C.byref(d), C.byref(slot)), allow=allow)
        if rc != OK:
            return None
        self.n_nodes[slot.value] = (n_side + 1) ** 3
        return slot.value

    def admit_prepared(self, prep, allow=()):
        """Admit a RunPrep (host part already done); None when it does not fit now."""
        slot = C.c_int(-1)
        rc = self._ck(self.L.mpg_batch_admit_prepared(self.h, prep.h, C.byref(slot)), allow=allow)
        if rc != OK:
            return None
        self.n_nodes[slot.value] = (prep.n_side + 1) ** 3
        return slot.value

    def step(self, n=1, allow=()):
        st = BatchStats()
        rc = self._ck(self.L.mpg_batch_step(self.h, n, C.byref(st)), allow=allow)
        st.rc = rc
        return st

    def info(self, slot):
        r = RunInfo()
        self._ck(self.L.mpg_batch_run_info(self.h, slot, C.byref(r)))
        return r

    def phi(self, slot):
        a = np.zeros(self.n_nodes[slot])
        self._ck(self.L.mpg_batch_run_phi(self.h, slot, ptr(a)))
        return a

    def particles(self, slot):
        n = C.c_int64()
        self._ck(self.L.mpg_batch_run_particles(self.h, slot, 0, C.byref(n), None, None, None), allow=(ERR_CAPACITY,))
        cap = max(n.value, 1)
        cell = np.zeros(cap, np.uint32)
        b = np.zeros((cap, 3), np.float32)
        v = np.zeros((cap, 3), np.float32)
        self._ck(self.L.mpg_batch_run_particles(self.h, slot, cap, C.byref(n), ptr(cell), ptr(b), ptr(v)))
        return cell[: n.value], b[: n.value], v[: n.value]

    def retire(self, slot):
        self._ck(self.L.mpg_batch_retire(self.h, slot))
        self.n_nodes.pop(slot, None)


class RunPrep:
    """The host part of a batch admission (mpg_batch_prepare): safe to build on
    any thread while another thread steps a batch."""

    def __init__(self, n_side, n_particles, seed, **kw):
        self.L = load()
        self.n_side = n_side
        d = Batch.desc(n_side, n_particles, seed, **kw)
        h = C.c_void_p()
        rc = self.L.mpg_batch_prepare(C.byref(d), C.byref(h))
        if rc != OK:
            raise MpgError(rc, "mpg_batch_prepare failed")
        self.h = h

    def close(self):
        if getattr(self, "h", None):
            self.L.mpg_run_prep_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass
