"""Problem generators (initial states on a uniform mesh, interior cells and faces).

Host-side counterparts of the reference's MeshBlock::ProblemGenerator hooks for the
workloads of this path:
  LinearWave    src/pgen/linear_wave.cpp (InitUserMeshData :76-186, ProblemGenerator
                :464-575, eigenvectors of Stone et al. 2008 as coded at :626-1010, L1 error
                of UserWorkAfterLoop :191-420)
  orszag_tang   src/pgen/orszag_tang.cpp:42-115
The arrays follow the reference layout (var, k, j, i) with i fastest; face fields are
(nx3, nx2, nx1+1), (nx3, nx2+1, nx1), (nx3+1, nx2, nx1).
"""
import math

import numpy as np

TINY = 1.0e-20


def _gen_rx(index, nrange):
    noffset = index - nrange // 2
    noffset_ceil = index - (nrange + 1) // 2
    return (noffset + noffset_ceil) / (2.0 * nrange)


def axis(nx, lo, hi):
    """Face and centre positions of a single-block axis (mesh/mesh.hpp:389-488,
    coordinates/coordinates.cpp:127-145, cartesian.cpp:29)."""
    xf = np.array([0.5 * (lo + hi) + (_gen_rx(i, nx) * hi - _gen_rx(i, nx) * lo)
                   for i in range(nx + 1)])
    xf[0], xf[-1] = lo, hi
    xv = 0.5 * (xf[1:] + xf[:-1])
    dx = (hi - lo) / nx
    return xf, xv, dx


class LinearWave:
    def __init__(self, nx, domain, mhd, gamma=1.666666666666667, amp=1.0e-6, wave_flag=0):
        self.nx, self.domain, self.mhd, self.amp, self.wf = nx, domain, mhd, amp, wave_flag
        self.gam = gamma
        gm1 = gamma - 1.0
        (x1a, x1b), (x2a, x2b), (x3a, x3b) = domain
        x1size, x2size, x3size = x1b - x1a, x2b - x2a, x3b - x3a
        ang_3 = math.atan(x1size / x2size)
        self.sin_a3, self.cos_a3 = math.sin(ang_3), math.cos(ang_3)
        ang_2 = math.atan(0.5 * (x1size * self.cos_a3 + x2size * self.sin_a3) / x3size)
        self.sin_a2, self.cos_a2 = math.sin(ang_2), math.cos(ang_2)
        x1 = x1size * self.cos_a2 * self.cos_a3
        x2 = x2size * self.cos_a2 * self.sin_a3
        x3 = x3size * self.sin_a2
        lam = x1
        if ang_3 != 0.0:
            lam = min(lam, x2)
        if ang_2 != 0.0:
            lam = min(lam, x3)
        self.k_par = 2.0 * math.pi / lam
        self.lam = lam
        d0, u0 = 1.0, 0.0
        self.d0, self.u0 = d0, u0
        self.bx0, self.by0, self.bz0 = 1.0, math.sqrt(2.0), 0.5
        self.p0 = 1.0 / gamma
        h0 = ((self.p0 / gm1 + 0.5 * d0 * (u0 * u0)) + self.p0) / d0
        if mhd:
            h0 += (self.bx0 ** 2 + self.by0 ** 2 + self.bz0 ** 2) / d0
        self.rem, self.ev = self._right_eigvec(d0, u0, h0, gm1)

    def _right_eigvec(self, d, v1, h, gm1):
        """Column wave_flag(=0) of the right eigenmatrix (eq. B3 hydro, B21 MHD)."""
        v2 = v3 = 0.0
        vsq = v1 * v1 + v2 * v2 + v3 * v3
        if not self.mhd:
            asq = gm1 * max((h - 0.5 * vsq), TINY)
            a = math.sqrt(asq)
            return [1.0, v1 - a, v2, v3, h - v1 * a], v1 - a
        x, y = 0.0, 1.0
        b1, b2, b3 = self.bx0, self.by0, self.bz0
        btsq = b2 * b2 + b3 * b3
        bt_starsq = (gm1 - (gm1 - 1.0) * y) * btsq
        vaxsq = b1 * b1 / d
        hp = h - (vaxsq + btsq / d)
        twid_asq = max((gm1 * (hp - 0.5 * vsq) - (gm1 - 1.0) * x), TINY)
        ct2 = bt_starsq / d
        tsum = vaxsq + ct2 + twid_asq
        tdif = vaxsq + ct2 - twid_asq
        cf2_cs2 = math.sqrt(tdif * tdif + 4.0 * twid_asq * ct2)
        cfsq = 0.5 * (tsum + cf2_cs2)
        cf = math.sqrt(cfsq)
        cssq = twid_asq * vaxsq / cfsq
        bt = math.sqrt(btsq)
        bt_star = math.sqrt(bt_starsq)
        bet2, bet3 = (1.0, 0.0) if bt == 0.0 else (b2 / bt, b3 / bt)
        bet2_star = bet2 / math.sqrt(gm1 - (gm1 - 1.0) * y)
        bet3_star = bet3 / math.sqrt(gm1 - (gm1 - 1.0) * y)
        bet_starsq = bet2_star * bet2_star + bet3_star * bet3_star
        vbet = v2 * bet2_star + v3 * bet3_star
        if (cfsq - cssq) == 0.0:
            alpha_f, alpha_s = 1.0, 0.0
        elif (twid_asq - cssq) <= 0.0:
            alpha_f, alpha_s = 0.0, 1.0
        elif (cfsq - twid_asq) <= 0.0:
            alpha_f, alpha_s = 1.0, 0.0
        else:
            alpha_f = math.sqrt((twid_asq - cssq) / (cfsq - cssq))
            alpha_s = math.sqrt((cfsq - twid_asq) / (cfsq - cssq))
        sqrtd = math.sqrt(d)
        isqrtd = 1.0 / sqrtd
        s = -1.0 if b1 < 0.0 else 1.0
        twid_a = math.sqrt(twid_asq)
        cs = math.sqrt(cssq)
        qs = cs * alpha_s * s
        as_prime = twid_a * alpha_s * isqrtd
        aspbb = as_prime * bt_star * bet_starsq
        ev0 = v1 - cf
        col = [alpha_f, alpha_f * ev0, alpha_f * v2 + qs * bet2_star, alpha_f * v3 + qs * bet3_star,
               alpha_f * (hp - v1 * cf) + qs * vbet + aspbb, as_prime * bet2_star,
               as_prime * bet3_star]
        return col, ev0

    # ---------------------------------------------------------------------------------
    def _axes(self):
        nx1, nx2, nx3 = self.nx
        (x1a, x1b), (x2a, x2b), (x3a, x3b) = self.domain
        return axis(nx1, x1a, x1b), axis(nx2, x2a, x2b), axis(nx3, x3a, x3b)

    def _cons_analytic(self):
        """Cell-centre conserved state (and cell-centred B for MHD), :219-257."""
        (x1f, x1v, dx1), (x2f, x2v, dx2), (x3f, x3v, dx3) = self._axes()
        Z, Y, X = np.meshgrid(x3v, x2v, x1v, indexing="ij")
        x = self.cos_a2 * (X * self.cos_a3 + Y * self.sin_a3) + Z * self.sin_a2
        sn = np.sin(self.k_par * x)
        amp, r = self.amp, self.rem
        ca2, sa2, ca3, sa3 = self.cos_a2, self.sin_a2, self.cos_a3, self.sin_a3
        d1 = self.d0 + amp * sn * r[0]
        mx = self.d0 * 0.0 + amp * sn * r[1]
        my = amp * sn * r[2]
        mz = amp * sn * r[3]
        u = np.empty((5,) + X.shape)
        u[0] = d1
        u[1] = mx * ca2 * ca3 - my * sa3 - mz * sa2 * ca3
        u[2] = mx * ca2 * sa3 + my * ca3 - mz * sa2 * sa3
        u[3] = mx * sa2 + mz * ca2
        gm1 = self.gam - 1.0
        e0 = self.p0 / gm1 + 0.5 * self.d0 * self.u0 * self.u0 + amp * sn * r[4]
        bcc = None
        if self.mhd:
            e0 = e0 + 0.5 * (self.bx0 ** 2 + self.by0 ** 2 + self.bz0 ** 2)
            bx = self.bx0
            by = self.by0 + amp * sn * r[5]
            bz = self.bz0 + amp * sn * r[6]
            bcc = np.empty((3,) + X.shape)
            bcc[0] = bx * ca2 * ca3 - by * sa3 - bz * sa2 * ca3
            bcc[1] = bx * ca2 * sa3 + by * ca3 - bz * sa2 * sa3
            bcc[2] = bx * sa2 + bz * ca2
        u[4] = e0
        return u, bcc

    def _A(self, comp, x1, x2, x3):
        """Vector potential components A1, A2, A3 (:588-624)."""
        ca2, sa2, ca3, sa3 = self.cos_a2, self.sin_a2, self.cos_a3, self.sin_a3
        kp = self.k_par
        dby = self.amp * self.rem[5]
        dbz = self.amp * self.rem[6]
        x = x1 * ca2 * ca3 + x2 * ca2 * sa3 + x3 * sa2
        y = -x1 * sa3 + x2 * ca3
        Az = -self.by0 * x + (dby / kp) * np.cos(kp * (x)) + self.bx0 * y
        if comp == 3:
            return Az * ca2
        Ay = self.bz0 * x - (dbz / kp) * np.cos(kp * (x))
        if comp == 1:
            return -Ay * sa3 - Az * sa2 * ca3
        return Ay * ca3 - Az * sa2 * sa3

    def initial_state(self):
        """Interior conserved state and face fields as the reference pgen sets them."""
        u, _ = self._cons_analytic()
        if not self.mhd:
            return u, None, None, None
        (x1f, x1v, dx1), (x2f, x2v, dx2), (x3f, x3v, dx3) = self._axes()
        # a1 on (x1v, x2f, x3f), a2 on (x1f, x2v, x3f), a3 on (x1f, x2f, x3v)
        Z, Y, X = np.meshgrid(x3f, x2f, x1v, indexing="ij")
        a1 = self._A(1, X, Y, Z)
        Z, Y, X = np.meshgrid(x3f, x2v, x1f, indexing="ij")
        a2 = self._A(2, X, Y, Z)
        Z, Y, X = np.meshgrid(x3v, x2f, x1f, indexing="ij")
        a3 = self._A(3, X, Y, Z)
        b1 = (a3[:, 1:, :] - a3[:, :-1, :]) / dx2 - (a2[1:, :, :] - a2[:-1, :, :]) / dx3
        b2 = (a1[1:, :, :] - a1[:-1, :, :]) / dx3 - (a3[:, :, 1:] - a3[:, :, :-1]) / dx1
        b3 = (a2[:, :, 1:] - a2[:, :, :-1]) / dx1 - (a1[:, 1:, :] - a1[:, :-1, :]) / dx2
        return u, np.ascontiguousarray(b1), np.ascontiguousarray(b2), np.ascontiguousarray(b3)

    def l1_errors(self, u, b1=None, b2=None, b3=None):
        """RMS of the per-variable L1 errors against the initial state (:298-372)."""
        ua, bcca = self._cons_analytic()
        (x1f, x1v, dx1), (x2f, x2v, dx2), (x3f, x3v, dx3) = self._axes()
        vol = dx1 * dx2 * dx3
        (x1a, x1b), (x2a, x2b), (x3a, x3b) = self.domain
        vdom = (x1b - x1a) * (x2b - x2a) * (x3b - x3a)
        l1 = [np.sum(np.abs(ua[n] - u[n]) * vol) / vdom for n in range(5)]
        if self.mhd:
            bc = [0.5 * b1[:, :, :-1] + 0.5 * b1[:, :, 1:], 0.5 * b2[:, :-1, :] + 0.5 * b2[:, 1:, :],
                  0.5 * b3[:-1, :, :] + 0.5 * b3[1:, :, :]]
            l1 += [np.sum(np.abs(bcca[n] - bc[n]) * vol) / vdom for n in range(3)]
        rms = math.sqrt(sum(e * e for e in l1))
        return rms, l1


def orszag_tang(nx, domain=((-0.5, 0.5), (-0.5, 0.5), (-0.5, 0.5)), gamma=5.0 / 3.0):
    """3-D (z-invariant) Orszag-Tang vortex from the vector potential
    A_z = B0/(4 pi) (cos 4 pi x - 2 cos 2 pi y), src/pgen/orszag_tang.cpp:42-115."""
    nx1, nx2, nx3 = nx
    (x1f, x1v, dx1), (x2f, x2v, dx2), (x3f, x3v, dx3) = (
        axis(nx1, *domain[0]), axis(nx2, *domain[1]), axis(nx3, *domain[2]))
    PI = 3.1415926535897932
    TWO_PI = 6.2831853071795862
    gm1 = gamma - 1.0
    B0 = 1.0 / math.sqrt(4.0 * PI)
    d0 = 25.0 / (36.0 * PI)
    v0 = 1.0
    p0 = 5.0 / (12.0 * PI)
    az = B0 / (4.0 * PI) * (np.cos(4.0 * PI * x1f)[None, :] - 2.0 * np.cos(TWO_PI * x2f)[:, None])
    u = np.zeros((5, nx3, nx2, nx1))
    u[0] = d0
    u[1] = (d0 * v0 * np.sin(TWO_PI * x2v))[None, :, None]
    u[2] = (-d0 * v0 * np.sin(TWO_PI * x1v))[None, None, :]
    b1 = np.empty((nx3, nx2, nx1 + 1))
    b1[:] = ((az[1:, :] - az[:-1, :]) / dx2)[None]
    b2 = np.empty((nx3, nx2 + 1, nx1))
    b2[:] = ((az[:, :-1] - az[:, 1:]) / dx1)[None]
    b3 = np.zeros((nx3 + 1, nx2, nx1))
    bc1 = 0.5 * (b1[:, :, :-1] + b1[:, :, 1:])
    bc2 = 0.5 * (b2[:, :-1, :] + b2[:, 1:, :])
    bc3 = 0.5 * (b3[:-1, :, :] + b3[1:, :, :])
    u[4] = (p0 / gm1 + 0.5 * (bc1 ** 2 + bc2 ** 2 + bc3 ** 2)
            + 0.5 * (u[1] ** 2 + u[2] ** 2 + u[3] ** 2) / u[0])
    return u, b1, b2, b3


def turbulent_box(nx, seed=20261203, mach=5.0, beta=1.0, gamma=1.0001, kmin=1, kmax=4,
                  expo=-4.0, jeans_number=2.0, domain=((0.0, 1.0),) * 3):
    """Magnetised self-gravitating turbulent box (no reference problem generator: the
    reference's turbulence driver needs FFTW). rho = 1, p = 1/gamma (c_s = 1), uniform
    B along z with plasma beta = 2 p / B^2, and a seeded Gaussian random solenoidal
    velocity: independent complex Gaussian amplitudes on the integer wavevectors of the
    shells kmin <= |k| <= kmax (Hermitian, so the field is real) with |v_k|^2 ~ k^expo,
    projected divergence-free, synthesised by three separable 1-D sums (only the few
    hundred modes of the shells exist, so no full-grid transform is needed), mean removed
    and scaled to rms Mach number `mach`. Returns (u, b1, b2, b3, four_pi_G, sha256 of the
    velocity field), with G set for the Jeans number n_J = L / lambda_J,
    lambda_J = c_s sqrt(pi / (G rho)):  G = pi n_J^2 c_s^2 / (rho L^2)."""
    import hashlib
    n1, n2, n3 = nx
    rng = np.random.default_rng(seed)
    kr = np.arange(-kmax, kmax + 1)
    nk = kr.size
    K3, K2, K1 = np.meshgrid(kr, kr, kr, indexing="ij")
    kk = np.sqrt(K1 ** 2 + K2 ** 2 + K3 ** 2)
    shell = (kk >= kmin - 1e-9) & (kk <= kmax + 1e-9)
    amp = np.where(shell, np.where(kk > 0, kk, 1.0) ** (0.5 * expo), 0.0)
    vk = []
    for _ in range(3):
        a = (rng.standard_normal(kk.shape) + 1j * rng.standard_normal(kk.shape)) * amp
        a = 0.5 * (a + np.conj(a[::-1, ::-1, ::-1]))  # a(-k) = conj(a(k)): a real field
        vk.append(a)
    ksq = np.where(kk > 0, kk ** 2, 1.0)
    div = (K1 * vk[0] + K2 * vk[1] + K3 * vk[2]) / ksq
    vk = [vk[0] - K1 * div, vk[1] - K2 * div, vk[2] - K3 * div]

    def synth(a):
        # v(x3, x2, x1) = Re sum_k a(k) exp(2 pi i k.x), cell centres of the unit cube
        e1 = np.exp(2j * np.pi * np.outer(kr, (np.arange(n1) + 0.5) / n1))  # [nk, n1]
        e2 = np.exp(2j * np.pi * np.outer(kr, (np.arange(n2) + 0.5) / n2))
        e3 = np.exp(2j * np.pi * np.outer(kr, (np.arange(n3) + 0.5) / n3))
        t = np.einsum("cba,cz->zba", a, e3)                     # [n3, nk2, nk1]
        t = np.einsum("zba,by->zya", t, e2)                     # [n3, n2, nk1]
        try:  # the last sum is the large one: on the GPU when there is one
            import torch
            if torch.cuda.is_available():
                tt = torch.from_numpy(t).cuda()
                return (tt @ torch.from_numpy(e1).cuda()).real.cpu().numpy()
        except ImportError:
            pass
        out = np.empty((n3, n2, n1))
        for z in range(n3):                                     # [n2, nk1] @ [nk1, n1]
            out[z] = np.real(t[z] @ e1)
        return out

    v = [synth(a) for a in vk]
    v = [a - a.mean() for a in v]
    rms = math.sqrt(float(np.mean(v[0] ** 2 + v[1] ** 2 + v[2] ** 2)))
    cs = 1.0
    v = [a * (mach * cs / rms) for a in v]
    rho, p = 1.0, cs * cs / gamma
    b0 = math.sqrt(2.0 * p / beta)
    u = np.zeros((5, n3, n2, n1))
    u[0] = rho
    u[1], u[2], u[3] = rho * v[0], rho * v[1], rho * v[2]
    ke = 0.5 * rho * (v[0] ** 2 + v[1] ** 2 + v[2] ** 2)
    u[4] = p / (gamma - 1.0) + ke + 0.5 * b0 * b0
    b1 = np.zeros((n3, n2, n1 + 1))
    b2 = np.zeros((n3, n2 + 1, n1))
    b3 = np.full((n3 + 1, n2, n1), b0)
    L = domain[0][1] - domain[0][0]
    G = math.pi * jeans_number ** 2 * cs * cs / (rho * L * L)
    h = hashlib.sha256(np.ascontiguousarray(np.stack(v)).tobytes()).hexdigest()
    return u, b1, b2, b3, 4.0 * math.pi * G, h


def block_axis(level, lx, mesh_nx, nrb, nx, lo, hi):
    """Cell centres of block (level, lx) along one axis of a multi-level mesh: the uniform
    generator at the level's resolution with the block edges of Mesh::SetBlockSizeAndBoundaries
    (mesh/mesh.cpp:1675-1690, coordinates/coordinates.cpp:127-145, cartesian.cpp:29)."""
    nroot = mesh_nx << level
    nrbl = nrb << level

    def gx(index, nrange):
        rx = _gen_rx(index, nrange)
        return 0.5 * (lo + hi) + (rx * hi - rx * lo)

    xf = np.array([gx(t + lx * nx, nroot) for t in range(nx + 1)])
    xf[0] = lo if lx == 0 else gx(lx, nrbl)
    xf[-1] = hi if lx == nrbl - 1 else gx(lx + 1, nrbl)
    return 0.5 * (xf[1:] + xf[:-1])


def blast_blocks(leaves, mesh_nx, block_nx, domain=((-1.0, 1.0),) * 3, gamma=5.0 / 3.0,
                 radius=0.1, pamb=0.1, prat=100.0, damb=1.0, drat=1.0, b0=1.0, angle=45.0,
                 mhd=True):
    """Spherical (M)HD blast wave, src/pgen/blast.cpp:54-211 (Cartesian, no ramp), per block
    of a multi-level mesh: dict (level, lx1, lx2, lx3) -> (u, b1, b2, b3) interiors."""
    nrb = [mesh_nx[d] // block_nx[d] for d in range(3)]
    ang = (math.pi / 180.0) * angle
    gm1 = gamma - 1.0
    out = {}
    n1, n2, n3 = block_nx
    for leaf in leaves:
        level = leaf[0]
        xv = [block_axis(level, leaf[1 + d], mesh_nx[d], nrb[d], block_nx[d], *domain[d])
              for d in range(3)]
        Z, Y, X = np.meshgrid(xv[2], xv[1], xv[0], indexing="ij")
        rad = np.sqrt((X - 0.0) ** 2 + (Y - 0.0) ** 2 + (Z - 0.0) ** 2)
        inside = rad < radius
        u = np.zeros((5, n3, n2, n1))
        u[0] = np.where(inside, drat * damb, damb)
        u[4] = np.where(inside, prat * pamb, pamb) / gm1
        b1 = b2 = b3 = None
        if mhd:
            b1 = np.full((n3, n2, n1 + 1), b0 * math.cos(ang))
            b2 = np.full((n3, n2 + 1, n1), b0 * math.sin(ang))
            b3 = np.zeros((n3 + 1, n2, n1))
            u[4] += 0.5 * b0 * b0
        out[tuple(leaf)] = (u, b1, b2, b3)
    return out
