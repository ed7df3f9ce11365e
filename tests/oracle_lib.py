"""ctypes binding to the CPU oracle (oracle/athena_oracle.c, oracle/mg_oracle.c,
oracle/fft_oracle.cpp) and helpers to run the reference solver on a seeded state.

Test infrastructure only: used by tests/, __graft_entry__.smoke() and bench.py's
CPU-baseline leg as the checker, never by the product path.
"""
import ctypes as C
import os
import subprocess

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
ORACLE_DIR = os.path.join(ROOT, "oracle")
LIB_PATH = os.path.join(ORACLE_DIR, "liboracle.so")
FFT_LIB_PATH = os.path.join(ORACLE_DIR, "liboracle_fft.so")

SOLVERS = {"hlle": 0, "hllc": 1, "hlld": 2, "lhllc": 3, "lhlld": 4}
INTEGRATORS = {"vl2": 0, "rk1": 1, "rk2": 2, "rk3": 3}
FLOOR = float(np.sqrt(1024 * np.finfo(np.float32).tiny))  # eos/adiabatic_mhd.cpp:29-30


class OrcParams(C.Structure):
    _fields_ = [("nx1", C.c_int), ("nx2", C.c_int), ("nx3", C.c_int), ("ng", C.c_int),
                ("mhd", C.c_int), ("rsolver", C.c_int), ("xorder", C.c_int),
                ("integrator", C.c_int),
                ("gamma", C.c_double), ("dfloor", C.c_double), ("pfloor", C.c_double),
                ("cfl", C.c_double),
                ("x1min", C.c_double), ("x1max", C.c_double), ("x2min", C.c_double),
                ("x2max", C.c_double), ("x3min", C.c_double), ("x3max", C.c_double)]


class MgParams(C.Structure):
    _fields_ = [("lmax", C.c_int), ("xmin", C.c_double * 3), ("xmax", C.c_double * 3),
                ("bc", C.c_int * 6), ("mporder", C.c_int), ("autompo", C.c_int),
                ("nodipole", C.c_int), ("mporigin", C.c_double * 3), ("fmg", C.c_int),
                ("eps", C.c_double), ("niter", C.c_int), ("omega", C.c_double)]


MG_BC = {"periodic": 0, "zerograd": 1, "zerofixed": 2, "multipole": 3}


def build_fft_oracle(force=False):
    """The C++ restatement of the turbulence driver and FFT gravity (std::random engines)."""
    src = os.path.join(ORACLE_DIR, "fft_oracle.cpp")
    if not force and os.path.exists(FFT_LIB_PATH) and \
            os.path.getmtime(FFT_LIB_PATH) > os.path.getmtime(src):
        return FFT_LIB_PATH
    subprocess.run(["g++", "-O2", "-std=c++17", "-ffp-contract=off", "-fPIC", "-shared", "-o",
                    FFT_LIB_PATH, src], check=True)
    return FFT_LIB_PATH


def build_oracle(force=False):
    """Compile the oracle with the flags that keep its FP64 arithmetic reproducible."""
    build_fft_oracle(force)
    src = os.path.join(ORACLE_DIR, "athena_oracle.c")
    if (not force and os.path.exists(LIB_PATH)
            and os.path.getmtime(LIB_PATH) > max(os.path.getmtime(src), os.path.getmtime(
                os.path.join(ORACLE_DIR, "mg_oracle.c")))):
        return LIB_PATH
    srcs = [src, os.path.join(ORACLE_DIR, "mg_oracle.c")]
    cmd = ["gcc", "-O3", "-std=c11", "-ffp-contract=off", "-fopenmp", "-fPIC", "-shared",
           "-o", LIB_PATH] + srcs + ["-lm"]
    subprocess.run(cmd, check=True)
    return LIB_PATH


_lib = None


def lib():
    global _lib
    if _lib is None:
        build_oracle()
        L = C.CDLL(LIB_PATH)
        L.orc_create.restype = C.c_void_p
        L.orc_create.argtypes = [C.POINTER(OrcParams)]
        L.orc_destroy.argtypes = [C.c_void_p]
        L.orc_dims.argtypes = [C.c_void_p, C.POINTER(C.c_int64)]
        L.orc_array.restype = C.POINTER(C.c_double)
        L.orc_array.argtypes = [C.c_void_p, C.c_int]
        L.orc_initialize.argtypes = [C.c_void_p, C.c_double]
        L.orc_cycle.argtypes = [C.c_void_p, C.c_int, C.c_double]
        L.orc_run.restype = C.c_int
        L.orc_run.argtypes = [C.c_void_p, C.c_double, C.c_int]
        L.orc_get_dt.restype = C.c_double
        L.orc_get_dt.argtypes = [C.c_void_p]
        L.orc_set_dt.argtypes = [C.c_void_p, C.c_double]
        L.orc_get_time.restype = C.c_double
        L.orc_get_time.argtypes = [C.c_void_p]
        L.orc_num_threads.restype = C.c_int
        L.orc_mg_create.restype = C.c_void_p
        L.orc_mg_create.argtypes = [C.POINTER(MgParams)]
        L.orc_mg_destroy.argtypes = [C.c_void_p]
        L.orc_mg_u.restype = C.POINTER(C.c_double)
        L.orc_mg_u.argtypes = [C.c_void_p]
        L.orc_mg_src.restype = C.POINTER(C.c_double)
        L.orc_mg_src.argtypes = [C.c_void_p]
        L.orc_mg_solve.argtypes = [C.c_void_p]
        L.orc_mg_vcycles.argtypes = [C.c_void_p, C.c_int]
        L.orc_mg_iterations.restype = C.c_int
        L.orc_mg_iterations.argtypes = [C.c_void_p]
        L.orc_mg_last_norm.restype = C.c_double
        L.orc_mg_last_norm.argtypes = [C.c_void_p]
        L.orc_mg_defect_norm.restype = C.c_double
        L.orc_mg_defect_norm.argtypes = [C.c_void_p]
        L.orc_mg_mpcoeff.argtypes = [C.c_void_p, C.POINTER(C.c_double)]
        L.orc_attach_gravity.restype = C.c_int
        L.orc_attach_gravity.argtypes = [C.c_void_p, C.c_void_p, C.c_double]
        L.orc_phi.restype = C.POINTER(C.c_double)
        L.orc_phi.argtypes = [C.c_void_p]
        _lib = L
    return _lib


class Oracle:
    """Single periodic block of nx1*nx2*nx3 cells (ghost width ng), FP64."""

    def __init__(self, nx, mhd, solver, xorder=2, integrator="vl2", gamma=5.0 / 3.0,
                 cfl=0.4, ng=2, domain=((0.0, 1.0), (0.0, 1.0), (0.0, 1.0)),
                 dfloor=FLOOR, pfloor=FLOOR):
        self.L = lib()
        p = OrcParams()
        p.nx1, p.nx2, p.nx3 = nx
        p.ng = ng
        p.mhd = int(mhd)
        p.rsolver = SOLVERS[solver]
        p.xorder = xorder
        p.integrator = INTEGRATORS[integrator]
        p.gamma = gamma
        p.dfloor, p.pfloor = dfloor, pfloor
        # VL2 in 3D limits the CFL number to 0.5 (time_integrator.cpp:216-218,887-896)
        lim = 0.5 if integrator == "vl2" else 1.0
        p.cfl = min(cfl, lim)
        (p.x1min, p.x1max), (p.x2min, p.x2max), (p.x3min, p.x3max) = domain
        self.p = p
        self.s = self.L.orc_create(C.byref(p))
        d = (C.c_int64 * 4)()
        self.L.orc_dims(self.s, d)
        self.n1, self.n2, self.n3, self.ncell = d[0], d[1], d[2], d[3]
        self.ng, self.nx, self.mhd = ng, tuple(nx), bool(mhd)

    def __del__(self):
        try:
            self.L.orc_destroy(self.s)
        except Exception:
            pass

    def _view(self, which, shape):
        ptr = self.L.orc_array(self.s, which)
        return np.ctypeslib.as_array(ptr, shape=shape)

    # arrays are re-fetched every time: the solver swaps register pointers
    @property
    def u(self):
        return self._view(0, (5, self.n3, self.n2, self.n1))

    @property
    def b1(self):
        return self._view(1, (self.n3, self.n2, self.n1 + 1))

    @property
    def b2(self):
        return self._view(2, (self.n3, self.n2 + 1, self.n1))

    @property
    def b3(self):
        return self._view(3, (self.n3 + 1, self.n2, self.n1))

    @property
    def w(self):
        return self._view(4, (5, self.n3, self.n2, self.n1))

    @property
    def bcc(self):
        return self._view(5, (3, self.n3, self.n2, self.n1))

    def interior_slices(self):
        g = self.ng
        nx1, nx2, nx3 = self.nx
        return slice(g, g + nx3), slice(g, g + nx2), slice(g, g + nx1)

    def load_interior(self, u, b1=None, b2=None, b3=None):
        """u: (5,nx3,nx2,nx1); b1: (nx3,nx2,nx1+1); b2: (nx3,nx2+1,nx1); b3: (nx3+1,nx2,nx1)."""
        g = self.ng
        nx1, nx2, nx3 = self.nx
        self.u[:, g:g + nx3, g:g + nx2, g:g + nx1] = u
        if self.mhd:
            self.b1[g:g + nx3, g:g + nx2, g:g + nx1 + 1] = b1
            self.b2[g:g + nx3, g:g + nx2 + 1, g:g + nx1] = b2
            self.b3[g:g + nx3 + 1, g:g + nx2, g:g + nx1] = b3

    def interior(self):
        g = self.ng
        nx1, nx2, nx3 = self.nx
        out = {"u": self.u[:, g:g + nx3, g:g + nx2, g:g + nx1].copy()}
        if self.mhd:
            out["b1"] = self.b1[g:g + nx3, g:g + nx2, g:g + nx1 + 1].copy()
            out["b2"] = self.b2[g:g + nx3, g:g + nx2 + 1, g:g + nx1].copy()
            out["b3"] = self.b3[g:g + nx3 + 1, g:g + nx2, g:g + nx1].copy()
        return out

    def attach_gravity(self, mg, four_pi_G):
        """Self-gravity through a multigrid oracle covering the same cubic mesh."""
        self._mg = mg  # keep the solver alive as long as the block uses it
        if self.L.orc_attach_gravity(self.s, mg.m, four_pi_G) != 0:
            raise ValueError("multigrid size differs from the mesh")

    @property
    def phi(self):
        return np.ctypeslib.as_array(self.L.orc_phi(self.s), shape=(self.n3, self.n2, self.n1))

    def initialize(self, tlim):
        self.L.orc_initialize(self.s, tlim)

    def cycle(self, n, tlim):
        self.L.orc_cycle(self.s, n, tlim)

    def run(self, tlim, nlim=-1):
        return self.L.orc_run(self.s, tlim, nlim)

    @property
    def dt(self):
        return self.L.orc_get_dt(self.s)

    @property
    def time(self):
        return self.L.orc_get_time(self.s)


class MgOracle:
    """FP64 multigrid on a cubic N^3 mesh (N = 2^lmax), one ghost layer per level."""

    def __init__(self, lmax, domain=((-0.5, 0.5),) * 3, bc="periodic", mporder=4, autompo=True,
                 nodipole=False, mporigin=(0.0, 0.0, 0.0), fmg=True, eps=-1.0, niter=10):
        self.L = lib()
        p = MgParams()
        p.lmax = lmax
        for d in range(3):
            p.xmin[d], p.xmax[d] = domain[d]
            p.mporigin[d] = mporigin[d]
        bcs = [bc] * 6 if isinstance(bc, str) else list(bc)
        for f in range(6):
            p.bc[f] = MG_BC[bcs[f]]
        p.mporder, p.autompo, p.nodipole = mporder, int(autompo), int(nodipole)
        p.fmg, p.eps, p.niter, p.omega = int(fmg), eps, niter, 1.15
        self.p = p
        self.m = self.L.orc_mg_create(C.byref(p))
        self.n = 1 << lmax

    def __del__(self):
        try:
            self.L.orc_mg_destroy(self.m)
        except Exception:
            pass

    def _view(self, ptr):
        nt = self.n + 2
        return np.ctypeslib.as_array(ptr, shape=(nt, nt, nt))

    @property
    def u(self):
        return self._view(self.L.orc_mg_u(self.m))

    @property
    def src(self):
        return self._view(self.L.orc_mg_src(self.m))

    def load_source(self, src_interior):
        self.src[1:-1, 1:-1, 1:-1] = src_interior

    def solve(self):
        self.L.orc_mg_solve(self.m)
        return self.L.orc_mg_iterations(self.m), self.L.orc_mg_last_norm(self.m)

    def vcycles(self, n):
        self.L.orc_mg_vcycles(self.m, n)

    def defect_norm(self):
        return self.L.orc_mg_defect_norm(self.m)

    def phi(self):
        return self.u[1:-1, 1:-1, 1:-1].copy()


# ------------------------------------------------------------------ seeded states ----
def smooth_random_state(nx, mhd, seed, amp=0.1, gamma=5.0 / 3.0):
    """A smooth, periodic, seeded state (a few random Fourier modes on a uniform
    background) with a divergence-free face field from a vector potential."""
    rng = np.random.default_rng(seed)
    nx1, nx2, nx3 = nx
    x = (np.arange(nx1) + 0.5) / nx1
    y = (np.arange(nx2) + 0.5) / nx2
    z = (np.arange(nx3) + 0.5) / nx3
    Z, Y, X = np.meshgrid(z, y, x, indexing="ij")

    def field(nm=3):
        f = np.zeros_like(X)
        for _ in range(nm):
            kx, ky, kz = rng.integers(-2, 3, size=3)
            ph = rng.uniform(0, 2 * np.pi)
            f += rng.uniform(-1, 1) * np.cos(2 * np.pi * (kx * X + ky * Y + kz * Z) + ph)
        return f

    rho = 1.0 + amp * field()
    v = [amp * field() for _ in range(3)]
    p = 1.0 / gamma + amp * 0.5 * field()
    u = np.empty((5, nx3, nx2, nx1))
    u[0] = rho
    for n in range(3):
        u[1 + n] = rho * v[n]
    ek = 0.5 * rho * (v[0] ** 2 + v[1] ** 2 + v[2] ** 2)
    u[4] = p / (gamma - 1.0) + ek
    if not mhd:
        return u, None, None, None
    # face fields = curl(A) + B0 on the staggered mesh (exactly divergence free)
    b0 = rng.uniform(0.3, 1.0, size=3)
    dx1, dx2, dx3 = 1.0 / nx1, 1.0 / nx2, 1.0 / nx3
    xf = np.arange(nx1 + 1) / nx1
    yf = np.arange(nx2 + 1) / nx2
    zf = np.arange(nx3 + 1) / nx3
    modes = [(rng.integers(1, 3, size=3), rng.uniform(0, 2 * np.pi, size=3),
              amp * rng.uniform(-0.5, 0.5, size=3)) for _ in range(2)]

    def A(comp, zz, yy, xx):
        a = 0.0
        for k, ph, am in modes:
            a = a + am[comp] * np.sin(2 * np.pi * (k[0] * xx + k[1] * yy + k[2] * zz) + ph[comp]) \
                / (2 * np.pi)
        return a

    # A1 on x1-edges (x1v, x2f, x3f), A2 on x2-edges (x1f, x2v, x3f), A3 on x3-edges
    Z1, Y1, X1 = np.meshgrid(zf, yf, x, indexing="ij")
    Z2, Y2, X2 = np.meshgrid(zf, y, xf, indexing="ij")
    Z3, Y3, X3 = np.meshgrid(z, yf, xf, indexing="ij")
    a1 = A(0, Z1, Y1, X1)  # (nx3+1, nx2+1, nx1)
    a2 = A(1, Z2, Y2, X2)  # (nx3+1, nx2, nx1+1)
    a3 = A(2, Z3, Y3, X3)  # (nx3, nx2+1, nx1+1)
    b1 = (a3[:, 1:, :] - a3[:, :-1, :]) / dx2 - (a2[1:, :, :] - a2[:-1, :, :]) / dx3 + b0[0]
    b2 = (a1[1:, :, :] - a1[:-1, :, :]) / dx3 - (a3[:, :, 1:] - a3[:, :, :-1]) / dx1 + b0[1]
    b3 = (a2[:, :, 1:] - a2[:, :, :-1]) / dx1 - (a1[:, 1:, :] - a1[:, :-1, :]) / dx2 + b0[2]
    # make the duplicated periodic faces exactly equal
    b1[:, :, -1] = b1[:, :, 0]
    b2[:, -1, :] = b2[:, 0, :]
    b3[-1, :, :] = b3[0, :, :]
    bc1 = 0.5 * (b1[:, :, :-1] + b1[:, :, 1:])
    bc2 = 0.5 * (b2[:, :-1, :] + b2[:, 1:, :])
    bc3 = 0.5 * (b3[:-1, :, :] + b3[1:, :, :])
    u[4] += 0.5 * (bc1 ** 2 + bc2 ** 2 + bc3 ** 2)
    return u, np.ascontiguousarray(b1), np.ascontiguousarray(b2), np.ascontiguousarray(b3)


def write_state(path, u, b1=None, b2=None, b3=None):
    with open(path, "wb") as f:
        f.write(np.ascontiguousarray(u, dtype="<f8").tobytes())
        if b1 is not None:
            for b in (b1, b2, b3):
                f.write(np.ascontiguousarray(b, dtype="<f8").tobytes())


def read_state(path, nx, mhd, phi=False):
    nx1, nx2, nx3 = nx
    raw = np.fromfile(path, dtype="<f8")
    hdr = raw[:3]
    o = 3
    n = 5 * nx1 * nx2 * nx3
    out = {"time": hdr[0], "dt": hdr[1], "ncycle": int(hdr[2]),
           "u": raw[o:o + n].reshape(5, nx3, nx2, nx1)}
    o += n
    if mhd:
        for key, shp in (("b1", (nx3, nx2, nx1 + 1)), ("b2", (nx3, nx2 + 1, nx1)),
                         ("b3", (nx3 + 1, nx2, nx1))):
            m = int(np.prod(shp))
            out[key] = raw[o:o + m].reshape(shp)
            o += m
    if phi:
        m = nx1 * nx2 * nx3
        out["phi"] = raw[o:o + m].reshape(nx3, nx2, nx1)
    return out


def athinput_text(nx, mb, domain, cfl, tlim, nlim, gamma, xorder, integrator, extra="",
                  blocks="", mesh_bc="periodic"):
    (x1a, x1b), (x2a, x2b), (x3a, x3b) = domain
    return f"""<job>
problem_id = st
<time>
cfl_number = {cfl!r}
nlim = {nlim}
tlim = {tlim!r}
integrator = {integrator}
xorder = {xorder}
ncycle_out = 100000
<mesh>
nx1 = {nx[0]}
x1min = {x1a!r}
x1max = {x1b!r}
ix1_bc = {mesh_bc}
ox1_bc = {mesh_bc}
nx2 = {nx[1]}
x2min = {x2a!r}
x2max = {x2b!r}
ix2_bc = {mesh_bc}
ox2_bc = {mesh_bc}
nx3 = {nx[2]}
x3min = {x3a!r}
x3max = {x3b!r}
ix3_bc = {mesh_bc}
ox3_bc = {mesh_bc}
<meshblock>
nx1 = {mb[0]}
nx2 = {mb[1]}
nx3 = {mb[2]}
<hydro>
gamma = {gamma!r}
<problem>
state_in = state_in.bin
state_out = state_out.bin
{extra}
{blocks}
"""


def run_reference_state(exe, workdir, nx, mb, mhd, u, b1, b2, b3, cfl, tlim, nlim,
                        gamma=5.0 / 3.0, xorder=2, integrator="vl2",
                        domain=((0.0, 1.0), (0.0, 1.0), (0.0, 1.0)), extra="", phi=False,
                        blocks="", mesh_bc="periodic"):
    """Run the reference binary built with the load_state harness pgen."""
    os.makedirs(workdir, exist_ok=True)
    write_state(os.path.join(workdir, "state_in.bin"), u, b1, b2, b3)
    with open(os.path.join(workdir, "athinput.st"), "w") as f:
        f.write(athinput_text(nx, mb, domain, cfl, tlim, nlim, gamma, xorder, integrator, extra,
                              blocks, mesh_bc))
    r = subprocess.run([exe, "-i", "athinput.st"], cwd=workdir, capture_output=True, text=True)
    if r.returncode != 0 or "FATAL" in r.stdout:
        raise RuntimeError("reference run failed:\n" + r.stdout[-2000:] + r.stderr[-2000:])
    return read_state(os.path.join(workdir, "state_out.bin"), nx, mhd, phi=phi)


_fft = None


def fft_lib():
    global _fft
    if _fft is None:
        build_fft_oracle()
        L = C.CDLL(FFT_LIB_PATH)
        L.orc_turb_create.restype = C.c_void_p
        L.orc_turb_create.argtypes = [C.c_int, C.c_int, C.c_int, C.POINTER(C.c_double),
                                      C.POINTER(C.c_int), C.POINTER(C.c_double), C.c_int64,
                                      C.c_double]
        L.orc_turb_destroy.argtypes = [C.c_void_p]
        L.orc_turb_drive.argtypes = [C.c_void_p, C.POINTER(C.c_double), C.c_double, C.c_double]
        L.orc_fft_gravity.argtypes = [C.c_int, C.c_int, C.c_int, C.POINTER(C.c_double),
                                      C.c_double, C.POINTER(C.c_double), C.POINTER(C.c_double)]
        _fft = L
    return _fft


def _d(a):
    return a.ctypes.data_as(C.POINTER(C.c_double))


class TurbOracle:
    """TurbulenceDriver on a mesh-wide interior state u[5][n3][n2][n1] (FP64)."""

    def __init__(self, n, lengths, turb_flag, dedt, rseed, nlow=0, nhigh=None, dtdrive=0.0,
                 tcorr=0.0, f_shear=-1.0, expo=2.0, time=0.0):
        self.n = tuple(n)
        nhigh = n[0] // 2 if nhigh is None else nhigh
        ln = np.asarray(lengths, dtype=np.float64)
        ic = (C.c_int * 3)(turb_flag, nlow, nhigh)
        dc = (C.c_double * 5)(dtdrive, tcorr, f_shear, expo, dedt)
        self.h = fft_lib().orc_turb_create(n[0], n[1], n[2], _d(ln), ic, dc, rseed, time)

    def drive(self, u, time, dt):
        """Driving at (time, dt) on a copy of u; returns the perturbed state."""
        u = np.array(u, dtype=np.float64, order="C", copy=True)
        fft_lib().orc_turb_drive(self.h, _d(u), time, dt)
        return u

    def close(self):
        if self.h:
            fft_lib().orc_turb_destroy(self.h)
            self.h = None

    def __del__(self):
        self.close()


def fft_gravity(rho, lengths, four_pi_G):
    """FFTGravityDriver::Solve on a periodic mesh: rho[n3][n2][n1] -> phi (same shape)."""
    rho = np.ascontiguousarray(rho, dtype=np.float64)
    n3, n2, n1 = rho.shape
    ln = np.asarray(lengths, dtype=np.float64)
    phi = np.zeros_like(rho)
    fft_lib().orc_fft_gravity(n1, n2, n3, _d(ln), four_pi_G, _d(rho), _d(phi))
    return phi
