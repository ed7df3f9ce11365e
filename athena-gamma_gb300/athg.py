"""ctypes binding of the C ABI in include/athena_gb300.h.

`Sim` holds one device context: a uniform periodic mesh of MeshBlocks in the block pool,
with helpers that move global interior arrays (reference AthenaArray layout, i fastest)
in and out. There is no CPU fallback: if the CUDA library cannot be loaded, or no GPU is
present, construction raises.
"""
import ctypes as C
import os

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "libathena_gb300.so")

HLLE, HLLC, HLLD, LHLLC, LHLLD = 0, 1, 2, 3, 4
SOLVERS = {"hlle": HLLE, "hllc": HLLC, "hlld": HLLD, "lhllc": LHLLC, "lhlld": LHLLD}
INTEGRATORS = {"vl2": 0, "rk1": 1, "rk2": 2, "rk3": 3}
PRECISIONS = {"fp64": 0, "mixed": 1, "dfloat": 2}
VAR_CONS, VAR_B1F, VAR_B2F, VAR_B3F, VAR_PRIM, VAR_BCC, VAR_PHI = range(7)
# default density/pressure floors of the reference EOS: sqrt(1024*FLT_MIN)
FLOOR = float(np.sqrt(1024 * np.finfo(np.float32).tiny))
# 3-D CFL limits of the integrators (reference task_list/time_integrator.cpp:216-218 etc.)
CFL_LIMIT = {"vl2": 0.5, "rk1": 1.0, "rk2": 1.0, "rk3": 1.0}

# names the C ABI exports (checked by the CPU tests against include/athena_gb300.h)
EXPORTS = [
    "athg_create", "athg_destroy", "athg_set_blocks", "athg_set_uniform_mesh",
    "athg_num_blocks", "athg_block_location", "athg_var_size", "athg_upload",
    "athg_download", "athg_initialize", "athg_stage", "athg_end_cycle", "athg_cycles",
    "athg_get_time", "athg_set_time", "athg_synchronize", "athg_stream",
    "athg_launches_per_cycle", "athg_calculate_fluxes", "athg_compute_corner_e",
    "athg_integrate", "athg_exchange_ghosts", "athg_conserved_to_primitive",
    "athg_new_block_dt", "athg_max_div_b", "athg_sum_conserved", "athg_last_error",
    "athg_mg_create", "athg_mg_destroy", "athg_mg_load_source", "athg_mg_set_phi",
    "athg_mg_solve", "athg_mg_vcycles", "athg_mg_defect_norm", "athg_mg_get_phi",
    "athg_mg_stream", "athg_mg_multipole", "athg_attach_gravity", "athg_history",
    "athg_get_tuning", "athg_set_tuning",
    "athg_block_cfl_dt_noalloc", "athg_set_refined_mesh", "athg_set_multilevel_blocks",
    "athg_smr_stats", "athg_resume", "athg_cycle_timing", "athg_amr_enable",
    "athg_amr_regrid", "athg_turb_attach", "athg_turb_drive", "athg_attach_fft_gravity",
    "athg_set_stage_kernel", "athg_get_stage_kernel",
]
MG_BC = {"periodic": 0, "zerograd": 1, "zerofixed": 2, "multipole": 3}


class MgConfig(C.Structure):
    _fields_ = [("nx", C.c_int), ("x1min", C.c_double), ("x1max", C.c_double),
                ("x2min", C.c_double), ("x2max", C.c_double), ("x3min", C.c_double),
                ("x3max", C.c_double), ("bc", C.c_int * 6), ("mporder", C.c_int),
                ("auto_mporigin", C.c_int), ("nodipole", C.c_int), ("mporigin", C.c_double * 3),
                ("mode", C.c_int), ("threshold", C.c_double), ("niteration", C.c_int),
                ("precision", C.c_int)]


class Config(C.Structure):
    _fields_ = [("nx1", C.c_int), ("nx2", C.c_int), ("nx3", C.c_int), ("nghost", C.c_int),
                ("magnetic", C.c_int), ("rsolver", C.c_int), ("xorder", C.c_int),
                ("integrator", C.c_int), ("precision", C.c_int),
                ("gamma", C.c_double), ("dfloor", C.c_double), ("pfloor", C.c_double),
                ("cfl_number", C.c_double), ("tlim", C.c_double)]


class Mesh(C.Structure):
    _fields_ = [("nx1", C.c_int), ("nx2", C.c_int), ("nx3", C.c_int),
                ("x1min", C.c_double), ("x1max", C.c_double), ("x2min", C.c_double),
                ("x2max", C.c_double), ("x3min", C.c_double), ("x3max", C.c_double),
                ("periodic", C.c_int * 3)]


class Region(C.Structure):
    _fields_ = [("x1min", C.c_double), ("x1max", C.c_double), ("x2min", C.c_double),
                ("x2max", C.c_double), ("x3min", C.c_double), ("x3max", C.c_double),
                ("level", C.c_int)]


class AmrConfig(C.Structure):
    _fields_ = [("threshold", C.c_double), ("deref_fraction", C.c_double),
                ("max_level", C.c_int), ("derefine_count", C.c_int)]


class TurbConfig(C.Structure):
    _fields_ = [("turb_flag", C.c_int), ("rseed", C.c_int64), ("nlow", C.c_int),
                ("nhigh", C.c_int), ("dtdrive", C.c_double), ("tcorr", C.c_double),
                ("f_shear", C.c_double), ("expo", C.c_double), ("dedt", C.c_double)]


class AthgError(RuntimeError):
    pass


_lib = None


def lib():
    """Load the CUDA library (built in-tree by __graft_entry__.build())."""
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(LIB_PATH):
        raise AthgError("CUDA library not built: %s (run __graft_entry__.build())" % LIB_PATH)
    L = C.CDLL(LIB_PATH)
    vp, i, d, sz = C.c_void_p, C.c_int, C.c_double, C.c_size_t
    L.athg_last_error.restype = C.c_char_p
    sig = {
        "athg_create": [C.POINTER(Config), C.POINTER(vp)],
        "athg_destroy": [vp],
        "athg_set_uniform_mesh": [vp, C.POINTER(Mesh)],
        "athg_num_blocks": [vp, C.POINTER(i)],
        "athg_block_location": [vp, i, C.POINTER(C.c_int64)],
        "athg_var_size": [vp, i, C.POINTER(sz)],
        "athg_upload": [vp, i, i, C.POINTER(d), sz],
        "athg_download": [vp, i, i, C.POINTER(d), sz],
        "athg_initialize": [vp],
        "athg_stage": [vp, i],
        "athg_end_cycle": [vp],
        "athg_cycles": [vp, i],
        "athg_get_time": [vp, C.POINTER(d), C.POINTER(d), C.POINTER(C.c_int64)],
        "athg_set_time": [vp, d, d, C.c_int64],
        "athg_synchronize": [vp],
        "athg_stream": [vp, C.POINTER(vp)],
        "athg_launches_per_cycle": [vp, C.POINTER(i)],
        "athg_calculate_fluxes": [vp, i],
        "athg_compute_corner_e": [vp],
        "athg_integrate": [vp, i],
        "athg_exchange_ghosts": [vp],
        "athg_conserved_to_primitive": [vp],
        "athg_new_block_dt": [vp, C.POINTER(d)],
        "athg_max_div_b": [vp, C.POINTER(d)],
        "athg_sum_conserved": [vp, C.POINTER(d)],
        "athg_mg_create": [C.POINTER(MgConfig), C.POINTER(vp)],
        "athg_mg_destroy": [vp],
        "athg_mg_load_source": [vp, C.POINTER(d), sz, d],
        "athg_mg_set_phi": [vp, C.POINTER(d), sz],
        "athg_mg_solve": [vp, C.POINTER(i), C.POINTER(d)],
        "athg_mg_vcycles": [vp, i],
        "athg_mg_defect_norm": [vp, C.POINTER(d)],
        "athg_mg_get_phi": [vp, C.POINTER(d), sz],
        "athg_mg_stream": [vp, C.POINTER(vp)],
        "athg_mg_multipole": [vp, C.POINTER(d)],
        "athg_attach_gravity": [vp, vp, d],
        "athg_history": [vp, C.POINTER(d), C.POINTER(i)],
        "athg_get_tuning": [vp, C.POINTER(i)],
        "athg_set_tuning": [vp, C.POINTER(i)],
        "athg_block_cfl_dt_noalloc": [C.POINTER(Config), vp, vp, vp, vp, vp, d, d, d, vp, vp],
        "athg_set_refined_mesh": [vp, C.POINTER(Mesh), i, C.POINTER(Region)],
        "athg_set_multilevel_blocks": [vp, C.POINTER(Mesh), i, C.POINTER(C.c_int64)],
        "athg_smr_stats": [vp, C.POINTER(C.c_int64)],
        "athg_resume": [vp],
        "athg_cycle_timing": [vp, i, C.POINTER(d), C.POINTER(i), C.c_char_p, sz],
        "athg_amr_enable": [vp, C.POINTER(AmrConfig)],
        "athg_amr_regrid": [vp, C.POINTER(i)],
        "athg_turb_attach": [vp, C.POINTER(Mesh), C.POINTER(TurbConfig)],
        "athg_turb_drive": [vp],
        "athg_attach_fft_gravity": [vp, C.POINTER(Mesh), d],
        "athg_set_stage_kernel": [vp, i, i],
        "athg_get_stage_kernel": [vp, C.POINTER(i), C.POINTER(i)],
    }
    for name, args in sig.items():
        f = getattr(L, name)
        f.argtypes = args
        f.restype = C.c_int
    _lib = L
    return L


def check(rc):
    if rc != 0:
        msg = lib().athg_last_error().decode(errors="replace")
        raise AthgError("athg error %d: %s" % (rc, msg))


def _dptr(a):
    return a.ctypes.data_as(C.POINTER(C.c_double))


class Sim:
    """A periodic mesh of MeshBlocks on the GPU: uniform, or refined by `regions`
    ([(x1min, x1max, x2min, x2max, x3min, x3max, level)]) or given as an explicit leaf list
    `leaves` ([(level, lx1, lx2, lx3)])."""

    def __init__(self, mesh_nx, block_nx, mhd, solver, precision="fp64", xorder=2,
                 integrator="vl2", gamma=5.0 / 3.0, cfl=0.4, tlim=1.0, ng=2,
                 domain=((0.0, 1.0), (0.0, 1.0), (0.0, 1.0)), dfloor=FLOOR, pfloor=FLOOR,
                 periodic=(1, 1, 1), regions=None, leaves=None):
        L = lib()
        c = Config()
        c.nx1, c.nx2, c.nx3 = block_nx
        c.nghost = ng
        c.magnetic = int(mhd)
        c.rsolver = SOLVERS[solver]
        c.xorder = xorder
        c.integrator = INTEGRATORS[integrator]
        c.precision = PRECISIONS[precision]
        c.gamma, c.dfloor, c.pfloor = gamma, dfloor, pfloor
        c.cfl_number = min(cfl, CFL_LIMIT[integrator])
        c.tlim = tlim
        self.cfg = c
        h = C.c_void_p()
        check(L.athg_create(C.byref(c), C.byref(h)))
        self.h = h
        m = Mesh()
        m.nx1, m.nx2, m.nx3 = mesh_nx
        (m.x1min, m.x1max), (m.x2min, m.x2max), (m.x3min, m.x3max) = domain
        for q in range(3):
            m.periodic[q] = int(periodic[q])
        if regions is not None:
            rs = (Region * max(1, len(regions)))()
            for q, r in enumerate(regions):
                rs[q].x1min, rs[q].x1max, rs[q].x2min, rs[q].x2max, rs[q].x3min, rs[q].x3max = r[:6]
                rs[q].level = int(r[6]) if len(r) > 6 else 1
            check(L.athg_set_refined_mesh(h, C.byref(m), len(regions), rs))
        elif leaves is not None:
            a = np.ascontiguousarray(np.asarray(leaves, dtype=np.int64).reshape(-1, 4))
            check(L.athg_set_multilevel_blocks(h, C.byref(m), a.shape[0],
                                               a.ctypes.data_as(C.POINTER(C.c_int64))))
        else:
            check(L.athg_set_uniform_mesh(h, C.byref(m)))
        self.mesh_nx, self.block_nx, self.ng, self.mhd = tuple(mesh_nx), tuple(block_nx), ng, mhd
        self._mesh = m
        self._list_blocks()
        self.multilevel = regions is not None or leaves is not None
        self.nc = tuple(n + 2 * ng for n in block_nx)

    def _list_blocks(self):
        L = lib()
        nb = C.c_int()
        check(L.athg_num_blocks(self.h, C.byref(nb)))
        self.nb = nb.value
        self.locs = []
        self.leaves = []  # (level, lx1, lx2, lx3) of every block
        loc = (C.c_int64 * 4)()
        for b in range(self.nb):
            check(L.athg_block_location(self.h, b, loc))
            self.locs.append((loc[0], loc[1], loc[2]))
            self.leaves.append((int(loc[3]), int(loc[0]), int(loc[1]), int(loc[2])))

    def amr_enable(self, threshold, max_level, derefine_count=10, deref_fraction=0.25):
        """Adaptive refinement with the blast criterion (athg_amr_enable); the block list
        (nb, leaves) is refreshed after every call that may regrid."""
        a = AmrConfig()
        a.threshold, a.deref_fraction = threshold, deref_fraction
        a.max_level, a.derefine_count = max_level, derefine_count
        check(lib().athg_amr_enable(self.h, C.byref(a)))
        self.multilevel = True
        self._list_blocks()

    def amr_regrid(self):
        """One refinement check and regrid; returns whether the mesh changed."""
        ch = C.c_int()
        check(lib().athg_amr_regrid(self.h, C.byref(ch)))
        self._list_blocks()
        return bool(ch.value)

    def close(self):
        if getattr(self, "h", None):
            lib().athg_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    # ---------------------------------------------------------------- layout ----
    def _shape(self, var):
        n1, n2, n3 = self.nc
        return {VAR_CONS: (5, n3, n2, n1), VAR_PRIM: (5, n3, n2, n1), VAR_BCC: (3, n3, n2, n1),
                VAR_B1F: (n3, n2, n1 + 1), VAR_B2F: (n3, n2 + 1, n1),
                VAR_B3F: (n3 + 1, n2, n1), VAR_PHI: (n3, n2, n1)}[var]

    def upload(self, var, blocks_array):
        a = np.ascontiguousarray(blocks_array, dtype=np.float64)
        check(lib().athg_upload(self.h, -1, var, _dptr(a), a.size))

    def download(self, var):
        shp = (self.nb,) + self._shape(var)
        a = np.empty(shp, dtype=np.float64)
        check(lib().athg_download(self.h, -1, var, _dptr(a), a.size))
        return a

    def load_interior(self, u, b1=None, b2=None, b3=None):
        """Scatter global interior arrays into the blocks (ghosts zero, filled later)."""
        g = self.ng
        nx1, nx2, nx3 = self.block_nx
        U = np.zeros((self.nb,) + self._shape(VAR_CONS))
        for b, (l1, l2, l3) in enumerate(self.locs):
            U[b, :, g:g + nx3, g:g + nx2, g:g + nx1] = \
                u[:, l3 * nx3:(l3 + 1) * nx3, l2 * nx2:(l2 + 1) * nx2, l1 * nx1:(l1 + 1) * nx1]
        self.upload(VAR_CONS, U)
        if self.mhd:
            B = [np.zeros((self.nb,) + self._shape(v)) for v in (VAR_B1F, VAR_B2F, VAR_B3F)]
            for b, (l1, l2, l3) in enumerate(self.locs):
                o1, o2, o3 = l1 * nx1, l2 * nx2, l3 * nx3
                B[0][b, g:g + nx3, g:g + nx2, g:g + nx1 + 1] = \
                    b1[o3:o3 + nx3, o2:o2 + nx2, o1:o1 + nx1 + 1]
                B[1][b, g:g + nx3, g:g + nx2 + 1, g:g + nx1] = \
                    b2[o3:o3 + nx3, o2:o2 + nx2 + 1, o1:o1 + nx1]
                B[2][b, g:g + nx3 + 1, g:g + nx2, g:g + nx1] = \
                    b3[o3:o3 + nx3 + 1, o2:o2 + nx2, o1:o1 + nx1]
            for v, arr in zip((VAR_B1F, VAR_B2F, VAR_B3F), B):
                self.upload(v, arr)

    def load_blocks(self, states):
        """Interior state per block: states[(level, lx1, lx2, lx3)] = (u, b1, b2, b3) in the
        interior layout (ghosts zero, filled by initialize())."""
        g = self.ng
        nx1, nx2, nx3 = self.block_nx
        U = np.zeros((self.nb,) + self._shape(VAR_CONS))
        B = [np.zeros((self.nb,) + self._shape(v)) for v in (VAR_B1F, VAR_B2F, VAR_B3F)]
        for b, key in enumerate(self.leaves):
            u, b1, b2, b3 = states[key]
            U[b, :, g:g + nx3, g:g + nx2, g:g + nx1] = u
            if self.mhd:
                B[0][b, g:g + nx3, g:g + nx2, g:g + nx1 + 1] = b1
                B[1][b, g:g + nx3, g:g + nx2 + 1, g:g + nx1] = b2
                B[2][b, g:g + nx3 + 1, g:g + nx2, g:g + nx1] = b3
        self.upload(VAR_CONS, U)
        if self.mhd:
            for v, arr in zip((VAR_B1F, VAR_B2F, VAR_B3F), B):
                self.upload(v, arr)

    def blocks(self, ghosts=True):
        """dict (level, lx1, lx2, lx3) -> {u, w, b1, b2, b3} (whole arrays with ghosts, or
        the interior)."""
        g = self.ng
        nx1, nx2, nx3 = self.block_nx
        arrs = {"u": self.download(VAR_CONS), "w": self.download(VAR_PRIM)}
        if self.mhd:
            arrs.update(b1=self.download(VAR_B1F), b2=self.download(VAR_B2F),
                        b3=self.download(VAR_B3F))
        out = {}
        for b, key in enumerate(self.leaves):
            d = {}
            for k, a in arrs.items():
                x = a[b]
                if not ghosts:
                    e1 = 1 if k == "b1" else 0
                    e2 = 1 if k == "b2" else 0
                    e3 = 1 if k == "b3" else 0
                    x = x[..., g:g + nx3 + e3, g:g + nx2 + e2, g:g + nx1 + e1]
                d[k] = x
            out[key] = d
        return out

    def cycle_timing(self):
        """One cycle launch group by launch group: [(name, ms)] in launch order."""
        ms = (C.c_double * 64)()
        n = C.c_int()
        buf = C.create_string_buffer(8192)
        check(lib().athg_cycle_timing(self.h, 64, ms, C.byref(n), buf, 8192))
        names = buf.value.decode().split("\n")
        return [(names[q], ms[q]) for q in range(n.value)]

    def smr_stats(self):
        out = (C.c_int64 * 8)()
        check(lib().athg_smr_stats(self.h, out))
        return tuple(out)

    def interior(self, prim=False):
        """Gather global interior arrays (u, and b1/b2/b3 for MHD)."""
        g = self.ng
        nx1, nx2, nx3 = self.block_nx
        N1, N2, N3 = self.mesh_nx
        U = self.download(VAR_PRIM if prim else VAR_CONS)
        u = np.empty((5, N3, N2, N1))
        for b, (l1, l2, l3) in enumerate(self.locs):
            u[:, l3 * nx3:(l3 + 1) * nx3, l2 * nx2:(l2 + 1) * nx2, l1 * nx1:(l1 + 1) * nx1] = \
                U[b, :, g:g + nx3, g:g + nx2, g:g + nx1]
        out = {"w" if prim else "u": u}
        if self.mhd and not prim:
            b1 = np.empty((N3, N2, N1 + 1))
            b2 = np.empty((N3, N2 + 1, N1))
            b3 = np.empty((N3 + 1, N2, N1))
            B1, B2, B3 = (self.download(v) for v in (VAR_B1F, VAR_B2F, VAR_B3F))
            for b, (l1, l2, l3) in enumerate(self.locs):
                o1, o2, o3 = l1 * nx1, l2 * nx2, l3 * nx3
                b1[o3:o3 + nx3, o2:o2 + nx2, o1:o1 + nx1 + 1] = B1[b, g:g + nx3, g:g + nx2, g:g + nx1 + 1]
                b2[o3:o3 + nx3, o2:o2 + nx2 + 1, o1:o1 + nx1] = B2[b, g:g + nx3, g:g + nx2 + 1, g:g + nx1]
                b3[o3:o3 + nx3 + 1, o2:o2 + nx2, o1:o1 + nx1] = B3[b, g:g + nx3 + 1, g:g + nx2, g:g + nx1]
            out.update(b1=b1, b2=b2, b3=b3)
        return out

    # ------------------------------------------------------------------ driver ----
    def initialize(self):
        check(lib().athg_initialize(self.h))

    def stage(self, s):
        check(lib().athg_stage(self.h, s))

    def end_cycle(self):
        check(lib().athg_end_cycle(self.h))

    def cycles(self, n):
        check(lib().athg_cycles(self.h, n))
        if self.multilevel:
            self._list_blocks()

    def synchronize(self):
        check(lib().athg_synchronize(self.h))

    def get_time(self):
        t, dt, n = C.c_double(), C.c_double(), C.c_int64()
        check(lib().athg_get_time(self.h, C.byref(t), C.byref(dt), C.byref(n)))
        return t.value, dt.value, n.value

    def set_time(self, time, dt, ncycle):
        check(lib().athg_set_time(self.h, time, dt, ncycle))

    def run(self, tlim, nlim=-1, chunk=1):
        """Whole cycles until time >= tlim (main.cpp:430 loop condition)."""
        n = 0
        t, _, _ = self.get_time()
        while t < tlim and (nlim < 0 or n < nlim):
            self.cycles(1)
            n += 1
            t, _, _ = self.get_time()
        return n

    def stream(self):
        s = C.c_void_p()
        check(lib().athg_stream(self.h, C.byref(s)))
        return s.value

    def launches_per_cycle(self):
        n = C.c_int()
        check(lib().athg_launches_per_cycle(self.h, C.byref(n)))
        return n.value

    def max_div_b(self):
        v = C.c_double()
        check(lib().athg_max_div_b(self.h, C.byref(v)))
        return v.value

    def sum_conserved(self):
        a = np.zeros(5)
        check(lib().athg_sum_conserved(self.h, _dptr(a)))
        return a

    def new_block_dt(self):
        v = C.c_double()
        check(lib().athg_new_block_dt(self.h, C.byref(v)))
        return v.value

    def tuning(self):
        """(x1 threads per block, marching threads per block, faces per segment)."""
        a = (C.c_int * 3)()
        check(lib().athg_get_tuning(self.h, a))
        return tuple(a)

    def set_tuning(self, x1_tpb, march_tpb, seg):
        a = (C.c_int * 3)(x1_tpb, march_tpb, seg)
        check(lib().athg_set_tuning(self.h, a))

    def set_stage_kernel(self, single, nseg=0):
        """Mixed VL2 MHD stage as one launch (single=True) or as separate sweeps; nseg
        k-segments per thread block of the single pass (0: autotuned)."""
        check(lib().athg_set_stage_kernel(self.h, int(bool(single)), int(nseg)))

    def stage_kernel(self):
        """(whether the next cycle runs the single-pass stage, its k-segments)."""
        a, b = C.c_int(), C.c_int()
        check(lib().athg_get_stage_kernel(self.h, C.byref(a), C.byref(b)))
        return bool(a.value), b.value

    def history(self):
        """The 12 history sums of outputs/history.cpp, reduced on the device."""
        a = np.zeros(12)
        n = C.c_int()
        check(lib().athg_history(self.h, _dptr(a), C.byref(n)))
        return a[:n.value]

    def attach_gravity(self, mg, four_pi_G):
        """Self-gravity through a Multigrid on the same mesh (None detaches)."""
        check(lib().athg_attach_gravity(self.h, mg.h if mg is not None else None, four_pi_G))
        self._grav = mg  # the solver must outlive the coupling

    def attach_fft_gravity(self, four_pi_G):
        """FFT self-gravity over the whole periodic mesh (0 detaches)."""
        check(lib().athg_attach_fft_gravity(self.h, C.byref(self._mesh), four_pi_G))
        self._grav = None

    def attach_turbulence(self, turb_flag, dedt, rseed=1, nlow=0, nhigh=None, dtdrive=0.0,
                          tcorr=0.0, f_shear=-1.0, expo=2.0):
        """The reference's turbulence driver (<problem> turb_flag, <turbulence> block);
        nhigh defaults to mesh nx1 / 2 as there; turb_flag 0 detaches."""
        if not turb_flag:
            check(lib().athg_turb_attach(self.h, C.byref(self._mesh), None))
            return
        t = TurbConfig()
        t.turb_flag, t.rseed, t.nlow = turb_flag, rseed, nlow
        t.nhigh = self.mesh_nx[0] // 2 if nhigh is None else nhigh
        t.dtdrive, t.tcorr, t.f_shear, t.expo, t.dedt = dtdrive, tcorr, f_shear, expo, dedt
        check(lib().athg_turb_attach(self.h, C.byref(self._mesh), C.byref(t)))

    def turb_drive(self):
        check(lib().athg_turb_drive(self.h))

    def phi(self):
        """Global potential with one ghost layer around the mesh: (N3+2, N2+2, N1+2)."""
        g = self.ng
        nx1, nx2, nx3 = self.block_nx
        N1, N2, N3 = self.mesh_nx
        P = self.download(VAR_PHI)
        out = np.zeros((N3 + 2, N2 + 2, N1 + 2))
        for b, (l1, l2, l3) in enumerate(self.locs):
            out[l3 * nx3:(l3 + 1) * nx3 + 2, l2 * nx2:(l2 + 1) * nx2 + 2,
                l1 * nx1:(l1 + 1) * nx1 + 2] = \
                P[b, g - 1:g + nx3 + 1, g - 1:g + nx2 + 1, g - 1:g + nx1 + 1]
        return out


class Multigrid:
    """Multigrid Poisson solver (lap phi = src) on a cubic mesh of nx^3 cells."""

    def __init__(self, nx, domain=((-0.5, 0.5),) * 3, bc="periodic", mporder=4,
                 auto_mporigin=True, nodipole=False, mporigin=(0.0, 0.0, 0.0), mode="FMG",
                 threshold=-1.0, niteration=10, precision="fp64"):
        L = lib()
        c = MgConfig()
        c.nx = nx
        (c.x1min, c.x1max), (c.x2min, c.x2max), (c.x3min, c.x3max) = domain
        bcs = [bc] * 6 if isinstance(bc, str) else list(bc)
        for f in range(6):
            c.bc[f] = MG_BC[bcs[f]]
        c.mporder, c.auto_mporigin, c.nodipole = mporder, int(auto_mporigin), int(nodipole)
        for q in range(3):
            c.mporigin[q] = mporigin[q]
        c.mode = 0 if mode.upper() == "FMG" else 1
        c.threshold, c.niteration = threshold, niteration
        c.precision = PRECISIONS[precision]
        h = C.c_void_p()
        check(L.athg_mg_create(C.byref(c), C.byref(h)))
        self.h, self.nx, self.cfg = h, nx, c

    def close(self):
        if getattr(self, "h", None):
            lib().athg_mg_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def load_source(self, rho, fac=1.0):
        a = np.ascontiguousarray(rho, dtype=np.float64)
        check(lib().athg_mg_load_source(self.h, _dptr(a), a.size, fac))

    def set_phi(self, phi):
        a = np.ascontiguousarray(phi, dtype=np.float64)
        check(lib().athg_mg_set_phi(self.h, _dptr(a), a.size))

    def solve(self):
        it, nrm = C.c_int(), C.c_double()
        check(lib().athg_mg_solve(self.h, C.byref(it), C.byref(nrm)))
        return it.value, nrm.value

    def vcycles(self, n):
        check(lib().athg_mg_vcycles(self.h, n))

    def defect_norm(self):
        v = C.c_double()
        check(lib().athg_mg_defect_norm(self.h, C.byref(v)))
        return v.value

    def phi(self):
        a = np.empty((self.nx,) * 3)
        check(lib().athg_mg_get_phi(self.h, _dptr(a), a.size))
        return a

    def stream(self):
        s = C.c_void_p()
        check(lib().athg_mg_stream(self.h, C.byref(s)))
        return s.value

    def multipole(self):
        a = np.zeros(28)
        check(lib().athg_mg_multipole(self.h, _dptr(a)))
        return a
