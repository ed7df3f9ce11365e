// athg_mg.cu -- multigrid Poisson solver on the GPU (C ABI in include/athena_gb300.h).
//
// A cubic mesh of N = 2^L cells per side is held as one device grid per level with one
// ghost layer; on such a mesh the reference's per-MeshBlock levels plus its root grid
// visit exactly these uniform levels (same stencils, colour parity, boundary fills,
// coarsest solve), so one launch covers a whole level. Reference routines:
//   smoother      gravity/mg_gravity.cpp:220-273     defect     :283-314
//   FAS rhs       gravity/mg_gravity.cpp:324-351     restrict   multigrid/multigrid.cpp:684-725
//   prolongation  multigrid/multigrid.cpp:733-832    FMG        :838-1048
//   cycles        multigrid/multigrid_driver.cpp:553-823, FAS with multipole faces :292-295
//   boundaries    bvals/cc/mg/bvals_mg.cpp:321-368, multigrid/mgbval_*.cpp
//   multipoles    multigrid/multigrid.cpp:1054-1300, multigrid_driver.cpp:1909-2018
//
// FP64 path: the reference's algorithm in FP64 (built without FMA contraction).
// Mixed path: FP32 FMG, then iterative refinement -- the FP64 defect of the FP64 solution
// drives an FP32 V(1,1) cycle on the correction equation (homogeneous boundaries), and
// the correction is accumulated in FP64 until the FP64 defect norm meets the threshold.
#include <cmath>
#include <cstring>
#include <string>
#include <vector>

#include "athena_gb300.h"
#include "athg_internal.h"
#include "athg_numeric.h"

namespace athg {
// the error channel of athg_last_error() (defined in athg_api.cu)
void set_last_error(const std::string& s);
}

namespace {

int mgfail(int code, const std::string& msg) {
  athg::set_last_error(msg);
  return code;
}
#define MCK(call)                                                                    \
  do {                                                                               \
    cudaError_t e_ = (call);                                                         \
    if (e_ != cudaSuccess)                                                           \
      return mgfail(ATHG_ERR_CUDA, std::string(#call) + ": " + cudaGetErrorString(e_)); \
  } while (0)
#define MCKL()                                                                       \
  do {                                                                               \
    cudaError_t e_ = cudaGetLastError();                                             \
    if (e_ != cudaSuccess)                                                           \
      return mgfail(ATHG_ERR_CUDA, std::string("kernel launch: ") + cudaGetErrorString(e_)); \
  } while (0)

constexpr int TPB = 256;
inline unsigned nblk(long long n) { return (unsigned)((n + TPB - 1) / TPB); }

__host__ __device__ inline long long ix(int nt, int k, int j, int i) {
  return ((long long)k * nt + j) * nt + i;
}

// ------------------------------------------------------------------------- kernels --
// Every level is n = 2^lg cells per side (a power of two is checked when the solver is
// made), so the kernels decode thread indices with shifts and masks: a division by a
// runtime n is a long instruction sequence, 64-bit ones longer still.
__device__ __forceinline__ int lg2(int n) { return __ffs(n) - 1; }

// With every face periodic and n even, a ghost cell holds a copy of the interior cell it
// wraps to, and that cell has the ghost's red-black colour. So a smoothing sweep can also
// write the periodic images of the cells it updates (push_images): it reads only cells of
// the other colour, so nothing it reads changes, and the level's ghost layer then needs no
// separate boundary fill.
template <typename T>
__device__ __forceinline__ void push_images(T* u, int n, int k, int j, int i, T v) {
  const int oi = i == 1 ? n + 1 : (i == n ? 0 : -1);
  const int oj = j == 1 ? n + 1 : (j == n ? 0 : -1);
  const int ok = k == 1 ? n + 1 : (k == n ? 0 : -1);
  if ((oi & oj & ok) == -1) return;  // not next to a face
  const int nt = n + 2;
  for (int s = 1; s < 8; ++s) {
    const int x = (s & 1) ? oi : i, y = (s & 2) ? oj : j, z = (s & 4) ? ok : k;
    if (x < 0 || y < 0 || z < 0) continue;
    u[ix(nt, z, y, x)] = v;
  }
}

// Red-black Gauss-Seidel half sweep: cells with (color + k + j + i - 1) even in the
// reference's local indexing (i = is + c, is + c + 2, ...), one thread per updated cell.
// Each kernel's per-cell work is a device function of the thread's index t, called by the
// kernel (one thread per index) and by k_vcycle_small (a block-strided loop per step).
template <typename T, typename I, bool PUSH = false>
__device__ __forceinline__ void smooth_cell(T* u, const T* src, int n, T dx2, T isix, int color,
                                            I t, int lg) {
  const int lh = lg > 0 ? lg - 1 : 0;  // (n + 1) / 2 = 2^lh cells of one colour per row
  const int ip = (int)(t & (I)((1 << lh) - 1));
  const I r = t >> lh;
  const int j = (int)(r & (I)(n - 1)) + 1;
  const int k = (int)(r >> lg) + 1;
  int c = (color + k + j) & 1;
  int i = 1 + c + 2 * ip;
  if (i > n) return;
  const int nt = n + 2;
  const long long q = ix(nt, k, j, i), sk = (long long)nt * nt, sj = nt;
  const T v = u[q] - ((T(6.0) * u[q] - u[q + sk] - u[q + sj] - u[q + 1] - u[q - sk] - u[q - sj] -
                       u[q - 1]) + src[q] * dx2) * isix;
  u[q] = v;
  if constexpr (PUSH) push_images(u, n, k, j, i, v);
}
__host__ __device__ inline long long smooth_count(int n) {
  return (long long)((n + 1) / 2) * n * n;
}
template <typename T, bool PUSH>
__global__ void k_smooth(T* __restrict__ u, const T* __restrict__ src, int n, T dx2, T isix,
                         int color) {
  long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  const long long cnt = smooth_count(n);
  if (t >= cnt) return;
  if (cnt <= 0x7fffffffLL)
    smooth_cell<T, int, PUSH>(u, src, n, dx2, isix, color, (int)t, lg2(n));
  else smooth_cell<T, long long, PUSH>(u, src, n, dx2, isix, color, t, lg2(n));
}

// interior cell (k, j, i) of an n^3 box (n = 2^lg) from a thread index t, i fastest
template <typename I>
__device__ __forceinline__ void box_cell(I t, int n, int lg, int& k, int& j, int& i) {
  i = (int)(t & (I)(n - 1)) + 1;
  j = (int)((t >> lg) & (I)(n - 1)) + 1;
  k = (int)(t >> (2 * lg)) + 1;
}

// defect of the fine level averaged onto the coarse cell (CalculateDefect + Restrict);
// with FAS the fine solution is restricted too (RestrictBlock).
template <typename T, typename I>
__device__ __forceinline__ void defect_restrict_cell(const T* uf, const T* sf, T* sc, T* uc, int nc,
                                                     T idx2, int fas, I t, int lg) {
  int i, j, k;
  box_cell(t, nc, lg, k, j, i);
  const int nf = 2 * nc, ntf = nf + 2, ntc = nc + 2;
  const long long sk = (long long)ntf * ntf, sj = ntf;
  const int fk = 2 * k - 1, fj = 2 * j - 1, fi = 2 * i - 1;
  T d[8];
  int q8 = 0;
  for (int dk = 0; dk < 2; ++dk)
    for (int dj = 0; dj < 2; ++dj)
      for (int di = 0; di < 2; ++di) {
        long long q = ix(ntf, fk + dk, fj + dj, fi + di);
        d[q8++] = (T(6.0) * uf[q] - uf[q + sk] - uf[q + sj] - uf[q + 1] - uf[q - sk] - uf[q - sj] -
                   uf[q - 1]) * idx2 + sf[q];
      }
  const long long qc = ix(ntc, k, j, i);
  sc[qc] = T(0.125) * (d[0] + d[1] + d[2] + d[3] + d[4] + d[5] + d[6] + d[7]);
  if (fas) {
    auto U = [&](int a, int b, int c) { return uf[ix(ntf, fk + a, fj + b, fi + c)]; };
    uc[qc] = T(0.125) * (U(0, 0, 0) + U(0, 0, 1) + U(0, 1, 0) + U(0, 1, 1) + U(1, 0, 0) +
                         U(1, 0, 1) + U(1, 1, 0) + U(1, 1, 1));
  }
}
template <typename T>
__global__ void k_defect_restrict(const T* __restrict__ uf, const T* __restrict__ sf,
                                  T* __restrict__ sc, T* __restrict__ uc, int nc, T idx2, int fas) {
  long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  const long long cnt = (long long)nc * nc * nc;
  if (t >= cnt) return;
  if (cnt <= 0x7fffffffLL)
    defect_restrict_cell<T, int>(uf, sf, sc, uc, nc, idx2, fas, (int)t, lg2(nc));
  else defect_restrict_cell<T, long long>(uf, sf, sc, uc, nc, idx2, fas, t, lg2(nc));
}

// plain 8-cell average (RestrictFMGSource)
template <typename T>
__global__ void k_restrict(const T* __restrict__ f, T* __restrict__ c, int nc) {
  long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= (long long)nc * nc * nc) return;
  int i, j, k;
  box_cell(t, nc, lg2(nc), k, j, i);
  const int ntf = 2 * nc + 2;
  const int fk = 2 * k - 1, fj = 2 * j - 1, fi = 2 * i - 1;
  auto F = [&](int a, int b, int cc) { return f[ix(ntf, fk + a, fj + b, fi + cc)]; };
  c[ix(nc + 2, k, j, i)] = T(0.125) * (F(0, 0, 0) + F(0, 0, 1) + F(0, 1, 0) + F(0, 1, 1) +
                                       F(1, 0, 0) + F(1, 0, 1) + F(1, 1, 0) + F(1, 1, 1));
}

// src -= L'(u) on the interior (CalculateFASRHS)
template <typename T, typename I>
__device__ __forceinline__ void fas_rhs_cell(const T* u, T* src, int n, T idx2, I t, int lg) {
  int i, j, k;
  box_cell(t, n, lg, k, j, i);
  const int nt = n + 2;
  const long long q = ix(nt, k, j, i), sk = (long long)nt * nt, sj = nt;
  src[q] -= (T(6.0) * u[q] - u[q + sk] - u[q + sj] - u[q + 1] - u[q - sk] - u[q - sj] - u[q - 1]) *
            idx2;
}
template <typename T>
__global__ void k_fas_rhs(const T* __restrict__ u, T* __restrict__ src, int n, T idx2) {
  long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  const long long cnt = (long long)n * n * n;
  if (t >= cnt) return;
  if (cnt <= 0x7fffffffLL) fas_rhs_cell<T, int>(u, src, n, idx2, (int)t, lg2(n));
  else fas_rhs_cell<T, long long>(u, src, n, idx2, t, lg2(n));
}

// trilinear prolongation of the coarse correction, added to the fine level
// (ProlongateAndCorrect); with FAS the correction is u_c - u_old_c.
template <typename T, typename I>
__device__ __forceinline__ void prolong_correct_cell(const T* uc, const T* uold, T* uf, int nc,
                                                     I t, int lg) {
  int i, j, k;
  box_cell(t, nc, lg, k, j, i);
  const int ntc = nc + 2, ntf = 2 * nc + 2;
  auto S = [&](int kk, int jj, int ii) -> T {
    long long q = ix(ntc, kk, jj, ii);
    return uold ? T(uc[q] - uold[q]) : uc[q];
  };
  const int fk = 2 * (k - 1) + 1, fj = 2 * (j - 1) + 1, fi = 2 * (i - 1) + 1;
  const T c0 = S(k, j, i);
  for (int oz = 0; oz < 2; ++oz)
    for (int oy = 0; oy < 2; ++oy)
      for (int ox = 0; ox < 2; ++ox) {
        const int dz = oz ? 1 : -1, dy = oy ? 1 : -1, dx = ox ? 1 : -1;
        uf[ix(ntf, fk + oz, fj + oy, fi + ox)] +=
            T(0.015625) * (T(27.0) * c0 + S(k + dz, j + dy, i + dx) +
                           T(9.0) * (S(k, j, i + dx) + S(k, j + dy, i) + S(k + dz, j, i)) +
                           T(3.0) * (S(k + dz, j + dy, i) + S(k + dz, j, i + dx) + S(k, j + dy, i + dx)));
      }
}
template <typename T>
__global__ void k_prolong_correct(const T* __restrict__ uc, const T* __restrict__ uold,
                                  T* __restrict__ uf, int nc) {
  long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  const long long cnt = (long long)nc * nc * nc;
  if (t >= cnt) return;
  if (cnt <= 0x7fffffffLL) prolong_correct_cell<T, int>(uc, uold, uf, nc, (int)t, lg2(nc));
  else prolong_correct_cell<T, long long>(uc, uold, uf, nc, t, lg2(nc));
}

// FMG prolongation: separable 1-D weights (5,30,-3)/32 per axis, 27 products summed in
// the reference's order, divided by 32768 (FMGProlongate)
template <typename T>
__global__ void k_fmg_prolong(const T* __restrict__ uc, T* __restrict__ uf, int nc) {
  long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= (long long)nc * nc * nc) return;
  int i, j, k;
  box_cell(t, nc, lg2(nc), k, j, i);
  const int ntc = nc + 2, ntf = 2 * nc + 2;
  T s[27];
  for (int a = 0; a < 3; ++a)
    for (int b = 0; b < 3; ++b)
      for (int c = 0; c < 3; ++c) s[(a * 3 + b) * 3 + c] = uc[ix(ntc, k - 1 + a, j - 1 + b, i - 1 + c)];
  const T w0[3] = {T(5.0), T(30.0), T(-3.0)}, w1[3] = {T(-3.0), T(30.0), T(5.0)};
  const int fk = 2 * (k - 1) + 1, fj = 2 * (j - 1) + 1, fi = 2 * (i - 1) + 1;
  for (int oz = 0; oz < 2; ++oz)
    for (int oy = 0; oy < 2; ++oy)
      for (int ox = 0; ox < 2; ++ox) {
        const T *wz = oz ? w1 : w0, *wy = oy ? w1 : w0, *wx = ox ? w1 : w0;
        T acc = (wz[0] * wy[0] * wx[0]) * s[0];
        for (int q = 1; q < 27; ++q) {
          int a = q / 9, b = (q / 3) % 3, c = q % 3;
          acc = acc + (wz[a] * wy[b] * wx[c]) * s[q];
        }
        uf[ix(ntf, fk + oz, fj + oy, fi + ox)] = acc / T(32768.0);
      }
}

struct MpCoef {
  double c[25];
  double o[3];
  int order;
};

__device__ double mp_phi(const MpCoef& m, double x, double y, double z) {
  const double* c = m.c;
  double x2 = x * x, y2 = y * y, z2 = z * z, xy = x * y, yz = y * z, zx = z * x;
  double r2 = x2 + y2 + z2;
  double ir2 = 1.0 / r2, ir1 = sqrt(ir2);
  double ir3 = ir2 * ir1, ir5 = ir3 * ir2;
  if (m.order == 2)
    return ir1 * c[0] + ir3 * (c[1] * y + c[2] * z + c[3] * x) +
           ir5 * (c[4] * xy + c[5] * yz + (3.0 * z2 - r2) * c[6] + c[7] * zx + c[8] * 0.5 * (x2 - y2));
  double ir7 = ir5 * ir2, ir9 = ir7 * ir2;
  double hx2my2 = 0.5 * (x2 - y2), x2mty2 = x2 - 3.0 * y2, tx2my2 = 3.0 * x2 - y2;
  return ir1 * c[0] + ir3 * (c[1] * y + c[2] * z + c[3] * x) +
         ir5 * (c[4] * xy + c[5] * yz + (3.0 * z2 - r2) * c[6] + c[7] * zx + c[8] * 0.5 * (x2 - y2)) +
         ir7 * (y * tx2my2 * c[9] + x * x2mty2 * c[15] + xy * z * c[10] + z * hx2my2 * c[14] +
                (5.0 * z2 - r2) * (y * c[11] + x * c[13]) + z * (z2 - 3.0 * r2) * c[12]) +
         ir9 * (xy * hx2my2 * c[16] + 0.125 * (x2 * x2mty2 - y2 * tx2my2) * c[24] +
                yz * tx2my2 * c[17] + zx * x2mty2 * c[23] +
                (7.0 * z2 - r2) * (xy * c[18] + hx2my2 * c[22]) +
                (7.0 * z2 - 3.0 * r2) * (yz * c[19] + zx * c[21]) +
                (35.0 * z2 * z2 - 30.0 * z2 * r2 + 3.0 * r2 * r2) * c[20]);
}

// level coordinates (multigrid/multigrid.cpp:1321-1346)
__device__ inline double xface(int i, int n, double lo, double hi) {
  if (i == 1) return lo;
  if (i == n + 1) return hi;
  return lo + (i - 1) * ((hi - lo) / n);
}
__device__ inline double xcen(int i, int n, double lo, double hi) {
  return 0.5 * (xface(i, n, lo, hi) + xface(i + 1, n, lo, hi));
}

// Boundary operation of each face (inner x1, outer x1, ..., outer x3)
enum FaceOp { OP_PERIODIC = 0, OP_COPY = 1, OP_NEGATE = 2, OP_MULTIPOLE = 3 };
struct FaceOps {
  int op[6];
  const double* tab;  // multipole faces: the expansion at each face's ghost positions
};

// The multipole expansion at the face positions of one level, for the six faces:
// tab[(2 ax + side) (n+2)^2 + a2 (n+2) + a1], (a1, a2) = (j, k) on x1 faces, (i, k) on x2
// faces and (i, j) on x3 faces (level coordinates of multigrid/multigrid.cpp:1321-1346;
// face-centre positions of bvals/cc/mg/bvals_mg.cpp:339-366 with
// multigrid/mgbval_multipole.cpp)
__global__ void k_mp_tab(double* tab, int n, double lo0, double hi0, double lo1, double hi1,
                         double lo2, double hi2, MpCoef mp) {
  const int nt = n + 2;
  const long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= 6LL * nt * nt) return;
  const int face = (int)(t / ((long long)nt * nt));
  const long long r = t % ((long long)nt * nt);
  const int a1 = (int)(r % nt), a2 = (int)(r / nt);
  const int ax = face >> 1, side = face & 1;
  double px, py, pz;
  if (ax == 0) {
    px = xface(side ? n + 1 : 1, n, lo0, hi0); py = xcen(a1, n, lo1, hi1); pz = xcen(a2, n, lo2, hi2);
  } else if (ax == 1) {
    px = xcen(a1, n, lo0, hi0); py = xface(side ? n + 1 : 1, n, lo1, hi1); pz = xcen(a2, n, lo2, hi2);
  } else {
    px = xcen(a1, n, lo0, hi0); py = xcen(a2, n, lo1, hi1); pz = xface(side ? n + 1 : 1, n, lo2, hi2);
  }
  tab[t] = mp_phi(mp, px - mp.o[0], py - mp.o[1], pz - mp.o[2]);
}

// Every ghost cell of one level in one launch. The reference fills periodic ghosts first,
// then the x1 faces, the x2 faces (over the x1 ghosts too) and the x3 faces (over all
// ghosts), each pass from the value inside its face (bvals/cc/mg/bvals_mg.cpp:321-368):
// zero gradient copies it, zero-fixed (and a multipole face in the homogeneous correction
// equation) negates it, a multipole face takes 2 phi_face - value. Composed per ghost cell:
// start from the interior cell its coordinates wrap (periodic axes) or mirror to, then apply
// the faces of its non-periodic ghost axes in x1, x2, x3 order, each with phi at the
// cell's own coordinates on earlier and periodic axes and the mirrored ones on later axes.
// Each ghost cell has one thread: the x1 faces take all of their (j, k), the x2 faces the
// interior i, the x3 faces the interior i and j.
__host__ __device__ inline long long shell_count(int n) {
  return 2LL * (n + 2) * (n + 2) + 2LL * n * (n + 2) + 2LL * n * n;
}
// P2 (the one-block levels, n = 2^lg <= 16): the quotients by n + 2 and (n + 2)^2 come
// from FP32 reciprocals (div_small; rnt = 1 / (n + 2), rnt2 = 1 / (n + 2)^2), the others
// from shifts.
template <typename T, bool P2 = false>
__device__ __forceinline__ void bc_shell_cell(T* a, int n, const FaceOps& f, int t, int lg = 0,
                                              float rnt = 0.0f, float rnt2 = 0.0f) {
  // the shell of a level up to n = 4096 has fewer than 2^31 cells
  const int nt = n + 2;
  const int nx1 = 2 * nt * nt, nx2 = 2 * n * nt, nx3 = 2 * n * n;
  int c[3];
  if (t < nx1) {
    const int side = P2 ? athg::div_small(t, rnt2) : t / (nt * nt);
    const int r = t - side * (nt * nt);
    const int rq = P2 ? athg::div_small(r, rnt) : r / nt;
    c[0] = side ? n + 1 : 0; c[1] = r - rq * nt; c[2] = rq;
  } else if ((t -= nx1) < nx2) {
    const int side = P2 ? athg::div_small(t >> lg, rnt) : t / (n * nt);
    const int r = t - side * (n * nt);
    const int rq = P2 ? (r >> lg) : r / n;
    c[1] = side ? n + 1 : 0; c[0] = 1 + (r - rq * n); c[2] = rq;
  } else if ((t -= nx2) < nx3) {
    const int side = P2 ? (t >> (2 * lg)) : t / (n * n);
    const int r = t - side * (n * n);
    const int rq = P2 ? (r >> lg) : r / n;
    c[2] = side ? n + 1 : 0; c[0] = 1 + (r - rq * n); c[1] = 1 + rq;
  } else {
    return;
  }
  int m[3];
  bool per[3];
#pragma unroll
  for (int d = 0; d < 3; ++d) {
    per[d] = f.op[2 * d] == OP_PERIODIC;
    const int x = c[d];
    m[d] = (x == 0) ? (per[d] ? n : 1) : (x == n + 1 ? (per[d] ? 1 : n) : x);
  }
  T v = a[ix(nt, m[2], m[1], m[0])];
#pragma unroll
  for (int d = 0; d < 3; ++d) {
    if (per[d] || (c[d] != 0 && c[d] != n + 1)) continue;
    const int side = c[d] == n + 1;
    const int op = f.op[2 * d + side];
    if (op == OP_NEGATE) {
      v = -v;
    } else if (op == OP_MULTIPOLE) {
      int q[3];
#pragma unroll
      for (int e = 0; e < 3; ++e) q[e] = (e < d || per[e]) ? c[e] : m[e];
      const int a1 = d == 0 ? q[1] : q[0], a2 = d == 2 ? q[1] : q[2];
      const double phi = f.tab[(long long)(2 * d + side) * nt * nt + (long long)a2 * nt + a1];
      v = (T)(2.0 * phi - (double)v);
    }
  }
  a[ix(nt, c[2], c[1], c[0])] = v;
}
template <typename T>
__global__ void k_bc_shell(T* a, int n, FaceOps f) {
  const long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= shell_count(n)) return;
  bc_shell_cell<T>(a, n, f, (int)t);
}

// ---- the coarse levels of a V-cycle in one thread block ----
// Levels 0..ls (at most kSmallLevels, n <= 16) are latency-bound: their ~60 launches of a
// few microseconds each become one launch. The block stages the levels' arrays in shared
// memory and runs, step after step with a barrier between them, exactly the sequence of
// vcycle() for those levels, down to the coarsest level's two smoothing sweeps
// (multigrid_driver.cpp:778-823, ni = 1 on a cubic power-of-two mesh), calling the same
// per-cell functions.
constexpr int kSmallLevels = 5;
constexpr int kSmallThreads = 1024;
template <typename T>
struct SmallV {
  T* u[kSmallLevels];
  T* src[kSmallLevels];
  T* uold[kSmallLevels];
  const double* tab[kSmallLevels];
  T dx2[kSmallLevels], idx2[kSmallLevels];
  int op[6];
  int ls, top, fas, subtract, coff;
  int push;    // every face periodic: the sweeps of levels L >= 1 write their ghost images
  int anyper;  // some face periodic
  T isix;
};

template <typename T>
__global__ void __launch_bounds__(kSmallThreads) k_vcycle_small(SmallV<T> v) {
  extern __shared__ unsigned char sm_raw[];
  T* sm = reinterpret_cast<T*>(sm_raw);
  T *u[kSmallLevels], *s[kSmallLevels], *o[kSmallLevels];
  long long off = 0;
  for (int L = 0; L <= v.ls; ++L) {
    const long long c = (long long)((1 << L) + 2) * ((1 << L) + 2) * ((1 << L) + 2);
    u[L] = sm + off; off += c;
    s[L] = sm + off; off += c;
    o[L] = nullptr;
    if (v.fas) { o[L] = sm + off; off += c; }
  }
  // every level here is n = 2^L <= 16: int indices, and the boundary fill's quotients by
  // n + 2 from FP32 reciprocals (bc_shell_cell's P2)
  const int tid = threadIdx.x, nth = blockDim.x;
  auto cells = [](int L) { return ((1 << L) + 2) * ((1 << L) + 2) * ((1 << L) + 2); };
  for (int L = 0; L <= v.ls; ++L)
    for (int q = tid; q < cells(L); q += nth) {
      u[L][q] = v.u[L][q];
      s[L][q] = v.src[L][q];
      if (v.fas) o[L][q] = v.uold[L][q];
    }
  __syncthreads();
  auto bc = [&](int L) {
    FaceOps f;
    for (int q = 0; q < 6; ++q) f.op[q] = v.op[q];
    f.tab = v.tab[L];
    const int n = 1 << L, nt = n + 2;
    const float rnt = 1.0f / (float)nt, rnt2 = 1.0f / (float)(nt * nt);
    for (int t = tid; t < (int)shell_count(n); t += nth)
      bc_shell_cell<T, true>(u[L], n, f, t, L, rnt, rnt2);
    __syncthreads();
  };
  // pushes and boundary fills between colour sweeps as in vcycle() (pushes, mid_fill)
  auto pushL = [&](int L) { return v.push && L >= 1; };
  auto midfill = [&](int L) { return v.anyper && !pushL(L); };
  auto smooth = [&](int L, int color) {
    const int n = 1 << L;
    if (pushL(L)) {
      for (int t = tid; t < (int)smooth_count(n); t += nth)
        smooth_cell<T, int, true>(u[L], s[L], n, v.dx2[L], v.isix, color ^ v.coff, t, L);
    } else {
      for (int t = tid; t < (int)smooth_count(n); t += nth)
        smooth_cell<T, int, false>(u[L], s[L], n, v.dx2[L], v.isix, color ^ v.coff, t, L);
    }
    __syncthreads();
  };
  auto store_old = [&](int L) {
    for (int q = tid; q < cells(L); q += nth) o[L][q] = u[L][q];
    __syncthreads();
  };
  auto fas_rhs = [&](int L) {
    const int n = 1 << L;
    for (int t = tid; t < n * n * n; t += nth)
      fas_rhs_cell<T, int>(u[L], s[L], n, v.idx2[L], t, L);
    __syncthreads();
  };
  auto zero = [&](int L) {
    for (int q = tid; q < cells(L); q += nth) u[L][q] = T(0.0);
    __syncthreads();
  };
  // down: vcycle() levels ls..1
  for (int L = v.ls; L > 0; --L) {
    // a level below the top was zeroed (ghosts included) unless FAS
    if (!(pushL(L) && !v.fas && L < v.top)) bc(L);
    if (v.fas && L < v.top) { store_old(L); fas_rhs(L); }
    smooth(L, 0);
    if (midfill(L)) bc(L);
    smooth(L, 1);
    if (!pushL(L)) bc(L);
    const int nc = 1 << (L - 1);
    for (int t = tid; t < nc * nc * nc; t += nth)
      defect_restrict_cell<T, int>(u[L], s[L], s[L - 1], u[L - 1], nc, v.idx2[L], v.fas, t,
                                         L - 1);
    __syncthreads();
    if (!v.fas) zero(L - 1);
  }
  // the coarsest level: with a mean to subtract its solution is zero
  if (v.subtract) {
    if (v.fas) { bc(0); store_old(0); }
    zero(0);
  } else {
    bc(0);
    if (v.fas) { store_old(0); fas_rhs(0); }
    smooth(0, 0);
    if (midfill(0)) bc(0);
    smooth(0, 1);
    bc(0);
  }
  // up: vcycle() levels 0..ls-1
  for (int L = 0; L < v.ls; ++L) {
    if (L == 0 || !pushL(L)) bc(L);
    const int nc = 1 << L;
    for (int t = tid; t < nc * nc * nc; t += nth)
      prolong_correct_cell<T, int>(u[L], v.fas ? o[L] : nullptr, u[L + 1], nc, t, L);
    __syncthreads();
    bc(L + 1);
    smooth(L + 1, 0);
    if (midfill(L + 1)) bc(L + 1);
    smooth(L + 1, 1);
  }
  for (int L = 0; L <= v.ls; ++L)
    for (int q = tid; q < cells(L); q += nth) {
      v.u[L][q] = u[L][q];
      v.src[L][q] = s[L][q];
      if (v.fas) v.uold[L][q] = o[L][q];
    }
}

template <typename T>
size_t small_smem(int ls, int fas) {
  size_t c = 0;
  for (int L = 0; L <= ls; ++L) c += (size_t)((1 << L) + 2) * ((1 << L) + 2) * ((1 << L) + 2);
  return c * (fas ? 3 : 2) * sizeof(T);
}

// ---- reductions (FP64 accumulation) ----
__device__ inline double warp_sum(double v) {
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  return v;
}
template <int NV>
__device__ void block_add(double (&v)[NV], double* out) {
  __shared__ double sh[NV][TPB / 32];
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  for (int q = 0; q < NV; ++q) {
    double s = warp_sum(v[q]);
    if (lane == 0) sh[q][w] = s;
  }
  __syncthreads();
  if (threadIdx.x < 32) {
    for (int q = 0; q < NV; ++q) {
      double s = (lane < TPB / 32) ? sh[q][lane] : 0.0;
      s = warp_sum(s);
      if (lane == 0) atomicAdd(out + q, s);
    }
  }
}

// the mean from the level sum, once (red[1] = red[0] * scale), so the passes that subtract
// it take one FP64 instruction per cell instead of two
__global__ void k_mean(double* red, double scale) { red[1] = red[0] * scale; }

template <typename T>
__global__ void k_sub_const(T* a, long long cnt, const double* ave) {
  long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= cnt) return;
  a[t] -= (T)(*ave);
}

// Column sums: one thread per (i, j) column and run of kColK cells along k, then one block
// reduction (a block reduction per cell cost more than the summed terms themselves).
constexpr int kColK = 32;
__host__ __device__ inline int col_chunks(int n) { return (n + kColK - 1) / kColK; }

// Sum of the interior cells of one level (Multigrid::CalculateTotal), as column sums.
template <typename T>
__global__ void k_sum(const T* a, int n, double* out) {
  long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  double v[1] = {0.0};
  if (t < (long long)n * n * col_chunks(n)) {
    const int lg = lg2(n);
    const int i = (int)(t & (n - 1)) + 1, j = (int)((t >> lg) & (n - 1)) + 1;
    const int k0 = 1 + (int)(t >> (2 * lg)) * kColK, k1 = min(n, k0 + kColK - 1);
    const long long sk = (long long)(n + 2) * (n + 2);
    const T* p = a + ix(n + 2, k0, j, i);
    double acc = 0.0;
    if constexpr (sizeof(T) == 4) {
      // FP32 values: the column as an unevaluated pair hi + lo of TwoSums (no FP64
      // instruction per cell), widened on the integer pipe and added once
      float hi = 0.0f, lo = 0.0f;
      for (int k = k0; k <= k1; ++k, p += sk) {
        float sum, err;
        athg::two_sum(hi, *p, sum, err);
        hi = sum;
        lo += err;
      }
      acc = athg::f2d_int(hi) + athg::f2d_int(lo);
    } else {
      for (int k = k0; k <= k1; ++k, p += sk) acc += (double)*p;
    }
    v[0] = acc;
  }
  block_add<1>(v, out);
}

// Sum of squared defects of the finest level, as column sums. FP64
// path: the FP64 defect. Mixed path (dfl): the seven-point sum exactly in integers and the
// rest in double-float, as k_defect_to32 forms it (the norm only steers the iteration).
__global__ void k_defect_sq(const double* u, const double* src, int n, double idx2,
                            float idx2_hi, float idx2_lo, int dfl, double* out) {
  long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  double v[1] = {0.0};
  if (t < (long long)n * n * col_chunks(n)) {
    const int lg = lg2(n);
    const int i = (int)(t & (n - 1)) + 1, j = (int)((t >> lg) & (n - 1)) + 1;
    const int k0 = 1 + (int)(t >> (2 * lg)) * kColK, k1 = min(n, k0 + kColK - 1);
    const int nt = n + 2;
    const long long sk = (long long)nt * nt, sj = nt;
    athg::ff acc = {0.0f, 0.0f};
    double accd = 0.0;
    for (int k = k0; k <= k1; ++k) {
      const long long q = ix(nt, k, j, i);
      if (dfl) {
        const double nb[6] = {u[q + sk], u[q - sk], u[q + sj], u[q - sj], u[q + 1], u[q - 1]};
        athg::ff lap;
        if (athg::lap7_ff(u[q], nb, lap)) {
          const athg::ff d = athg::ff_add(athg::ff_mul(lap, athg::ff{idx2_hi, idx2_lo}),
                                          athg::split_ff(src[q]));
          acc = athg::ff_add(acc, athg::ff_sqr(d));
          continue;
        }
      }
      const double d =
          (6.0 * u[q] - u[q + sk] - u[q + sj] - u[q + 1] - u[q - sk] - u[q - sj] - u[q - 1]) *
              idx2 + src[q];
      accd += d * d;
    }
    v[0] = accd + (athg::f2d_int(acc.hi) + athg::f2d_int(acc.lo));
  }
  block_add<1>(v, out);
}

// Defect of the FP64 solution, narrowed to the FP32 correction source (mixed path only).
// FP64 issues at 1/64 of the FP32 rate here, so the seven-point sum is formed exactly in
// 64-bit integers (athg::lap7_ff, more accurate than six FP64 roundings) and scaled and
// added to the source in double-float arithmetic; values outside the integer form's range
// (or not finite) take the FP64 formula.
__global__ void k_defect_to32(const double* u, const double* src, int n, double idx2,
                              float idx2_hi, float idx2_lo, float* r32) {
  long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= (long long)n * n * n) return;
  int i, j, k;
  box_cell(t, n, lg2(n), k, j, i);
  const int nt = n + 2;
  const long long q = ix(nt, k, j, i), sk = (long long)nt * nt, sj = nt;
  const double c = u[q];
  const double nb[6] = {u[q + sk], u[q - sk], u[q + sj], u[q - sj], u[q + 1], u[q - 1]};
  athg::ff lap;
  if (athg::lap7_ff(c, nb, lap)) {
    const athg::ff d = athg::ff_add(athg::ff_mul(lap, athg::ff{idx2_hi, idx2_lo}),
                                    athg::split_ff(src[q]));
    r32[q] = athg::ff_f(d);
  } else {
    const double s = ((nb[0] + nb[1]) + (nb[2] + nb[3])) + (nb[4] + nb[5]);
    r32[q] = athg::d2f_int(fma(fma(6.0, c, -s), idx2, src[q]));
  }
}

__global__ void k_add_correction(double* u, const float* e, long long cnt) {
  long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (t < cnt) u[t] += athg::f2d_int(e[t]);
}
__global__ void k_widen(const float* a, double* b, long long cnt) {
  long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (t < cnt) b[t] = athg::f2d_int(a[t]);
}
__global__ void k_narrow(const double* a, float* b, long long cnt) {
  long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (t < cnt) b[t] = athg::d2f_int(a[t]);
}
// the mean subtraction of the FP64 source (k_sub_const) and its narrowing in one pass
__global__ void k_sub_narrow(double* a, float* b, long long cnt, const double* ave) {
  long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= cnt) return;
  const double v = a[t] - *ave;
  a[t] = v;
  b[t] = athg::d2f_int(v);
}
// the widening of the FP32 FMG solution and its mean subtraction (k_sub_const) in one pass
__global__ void k_widen_sub(const float* a, double* b, long long cnt, const double* ave) {
  long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (t < cnt) b[t] = athg::f2d_int(a[t]) - *ave;
}

// multipole moments (and the centre of mass) of the finest source, FP64, as column sums (x
// and y fixed per thread): per-cell reductions of 25 sums cost ten times the moments.
__global__ void k_com(const double* src, int n, double lo0, double hi0, double lo1, double hi1,
                      double lo2, double hi2, double vol, double* out) {
  long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  double v[4] = {0, 0, 0, 0};
  if (t < (long long)n * n * col_chunks(n)) {
    const int lg = lg2(n);
    const int i = (int)(t & (n - 1)) + 1, j = (int)((t >> lg) & (n - 1)) + 1;
    const int k0 = 1 + (int)(t >> (2 * lg)) * kColK, k1 = min(n, k0 + kColK - 1);
    const double x = xcen(i, n, lo0, hi0), y = xcen(j, n, lo1, hi1);
    for (int k = k0; k <= k1; ++k) {
      const double s = src[ix(n + 2, k, j, i)] * vol;
      v[0] += s; v[1] += s * y; v[2] += s * xcen(k, n, lo2, hi2); v[3] += s * x;
    }
  }
  block_add<4>(v, out);
}

__global__ void k_moments(const double* src, int n, double lo0, double hi0, double lo1, double hi1,
                          double lo2, double hi2, double vol, const double* origin, int order,
                          int nodipole, double* out) {
  long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  double m[25];
  for (int q = 0; q < 25; ++q) m[q] = 0.0;
  if (t < (long long)n * n * col_chunks(n)) {
    const int lg = lg2(n);
    const int i = (int)(t & (n - 1)) + 1, j = (int)((t >> lg) & (n - 1)) + 1;
    const int k0 = 1 + (int)(t >> (2 * lg)) * kColK, k1 = min(n, k0 + kColK - 1);
    const double y = xcen(j, n, lo1, hi1) - origin[1], y2 = y * y;
    const double x = xcen(i, n, lo0, hi0) - origin[0];
    const double x2 = x * x, xy = x * y;
    for (int k = k0; k <= k1; ++k) {
      double z = xcen(k, n, lo2, hi2) - origin[2], z2 = z * z;
      double yz = y * z, zx = z * x;
      double r2 = x2 + y2 + z2;
      double s = src[ix(n + 2, k, j, i)] * vol;
      m[0] += s;
      if (!nodipole) { m[1] += s * y; m[2] += s * z; m[3] += s * x; }
      m[4] += s * xy; m[5] += s * yz; m[6] += s * (3.0 * z2 - r2); m[7] += s * zx;
      if (order == 4) {
        double hx2my2 = 0.5 * (x2 - y2), x2mty2 = x2 - 3.0 * y2, tx2my2 = 3.0 * x2 - y2;
        double fz2mr2 = 5.0 * z2 - r2, sz2mr2 = 7.0 * z2 - r2, sz2mtr2 = 7.0 * z2 - 3.0 * r2;
        m[8] += s * hx2my2;
        m[9] += s * y * tx2my2; m[10] += s * xy * z; m[11] += s * y * fz2mr2;
        m[12] += s * z * (z2 - 3.0 * r2); m[13] += s * x * fz2mr2; m[14] += s * z * hx2my2;
        m[15] += s * x * x2mty2; m[16] += s * xy * hx2my2; m[17] += s * yz * tx2my2;
        m[18] += s * xy * sz2mr2; m[19] += s * yz * sz2mtr2;
        m[20] += s * (35.0 * z2 * z2 - 30.0 * z2 * r2 + 3.0 * r2 * r2);
        m[21] += s * zx * sz2mtr2; m[22] += s * hx2my2 * sz2mr2; m[23] += s * zx * x2mty2;
        m[24] += s * 0.125 * (x2 * x2mty2 - y2 * tx2my2);
      } else {
        m[8] += s * 0.5 * (x2 - y2);
      }
    }
  }
  block_add<25>(m, out);
}

// --------------------------------------------------------------------- hierarchy --
template <typename T>
struct Hier {
  int nl = 0;
  std::vector<T*> u, src, uold;
  std::vector<int> n;
  std::vector<double> dx;
  std::vector<double*> mptab;  // multipole faces: the expansion at every level's faces
  size_t cells(int L) const { return (size_t)(n[L] + 2) * (n[L] + 2) * (n[L] + 2); }
  size_t faces(int L) const { return 6 * (size_t)(n[L] + 2) * (n[L] + 2); }
};

template <typename T>
int alloc_hier(Hier<T>& h, int lmax, double rdx, bool with_old) {
  h.nl = lmax + 1;
  h.u.assign(h.nl, nullptr); h.src.assign(h.nl, nullptr); h.uold.assign(h.nl, nullptr);
  h.n.resize(h.nl); h.dx.resize(h.nl);
  for (int L = 0; L < h.nl; ++L) {
    h.n[L] = 1 << L;
    // finest width scaled by powers of two, as the reference does for coarser levels
    h.dx[L] = rdx * (double)(1 << (lmax - L));
    size_t c = h.cells(L);
    MCK(cudaMalloc(&h.u[L], c * sizeof(T)));
    MCK(cudaMalloc(&h.src[L], c * sizeof(T)));
    MCK(cudaMemset(h.u[L], 0, c * sizeof(T)));
    MCK(cudaMemset(h.src[L], 0, c * sizeof(T)));
    if (with_old) {
      MCK(cudaMalloc(&h.uold[L], c * sizeof(T)));
      MCK(cudaMemset(h.uold[L], 0, c * sizeof(T)));
    }
  }
  return ATHG_OK;
}
// only the finest level's u and src are allocated
int alloc_top(Hier<double>& h, int lmax, double rdx) {
  h.nl = lmax + 1;
  h.u.assign(h.nl, nullptr); h.src.assign(h.nl, nullptr); h.uold.assign(h.nl, nullptr);
  h.n.resize(h.nl); h.dx.resize(h.nl);
  for (int L = 0; L < h.nl; ++L) {
    h.n[L] = 1 << L;
    h.dx[L] = rdx * (double)(1 << (lmax - L));
  }
  size_t c = h.cells(lmax);
  MCK(cudaMalloc(&h.u[lmax], c * sizeof(double)));
  MCK(cudaMalloc(&h.src[lmax], c * sizeof(double)));
  MCK(cudaMemset(h.u[lmax], 0, c * sizeof(double)));
  MCK(cudaMemset(h.src[lmax], 0, c * sizeof(double)));
  return ATHG_OK;
}

template <typename T>
void free_hier(Hier<T>& h) {
  for (auto* p : h.u) if (p) cudaFree(p);
  for (auto* p : h.src) if (p) cudaFree(p);
  for (auto* p : h.uold) if (p) cudaFree(p);
  for (auto* p : h.mptab) if (p) cudaFree(p);
  h.u.clear(); h.src.clear(); h.uold.clear(); h.mptab.clear();
}

}  // namespace

struct athg_mg {
  athg_mg_config cfg{};
  int lmax = 0;
  bool periodic = true, subtract = true, fas = false, any_mp = false;
  bool any_periodic = false;  // some face periodic
  double rdx = 0.0, vol = 0.0;
  cudaStream_t st = nullptr;
  cudaStream_t own_st = nullptr;  // the stream created with the solver
  Hier<double> h64;      // FP64 path: all levels; mixed path: finest level only
  Hier<float> h32;       // mixed path: FP32 hierarchy
  double* red = nullptr; // reduction scratch [0..31]
  double* mpo_d = nullptr;
  MpCoef mp{};
  int coffset = 0;       // colour offset, flipped at every V-cycle (multigrid_driver.cpp:686)
  int coffset32 = 0;
  int iterations = 0;
  double last_norm = 0.0;
  // one captured cycle per colour-offset parity (the kernels take colour ^ offset); the
  // multipole boundaries read the face tables, rewritten in place by every new expansion,
  // so the captured cycles stay valid from solve to solve
  cudaGraph_t cyc_graph[2] = {nullptr, nullptr};
  cudaGraphExec_t cyc_exec[2] = {nullptr, nullptr};
};

namespace {

#define RC(x) do { int r_ = (x); if (r_) return r_; } while (0)

// the boundary operation of each face; multipole faces need level L's face table
template <typename T>
int face_ops(athg_mg* m, Hier<T>& h, int L, bool homogeneous, FaceOps* f) {
  f->tab = nullptr;
  for (int q = 0; q < 6; ++q) {
    const int b = m->cfg.bc[q];
    if (b == ATHG_MG_PERIODIC) f->op[q] = OP_PERIODIC;
    else if (b == ATHG_MG_ZEROGRAD) f->op[q] = OP_COPY;
    else if (b == ATHG_MG_ZEROFIXED || homogeneous) f->op[q] = OP_NEGATE;
    else f->op[q] = OP_MULTIPOLE;
    if (f->op[q] == OP_MULTIPOLE) {
      if ((int)h.mptab.size() <= L || !h.mptab[L])
        return mgfail(ATHG_ERR_STATE, "multipole boundary without its face table");
      f->tab = h.mptab[L];
    }
  }
  return ATHG_OK;
}

template <typename T>
int apply_bc(athg_mg* m, Hier<T>& h, int L, bool homogeneous) {
  const int n = h.n[L];
  FaceOps f;
  RC(face_ops(m, h, L, homogeneous, &f));
  k_bc_shell<T><<<nblk(shell_count(n)), TPB, 0, m->st>>>(h.u[L], n, f);
  MCKL();
  return ATHG_OK;
}

// zeroed face tables of every level (multipole boundaries)
template <typename T>
int alloc_mptab(Hier<T>& h) {
  h.mptab.assign(h.nl, nullptr);
  for (int L = 0; L < h.nl; ++L) {
    MCK(cudaMalloc(&h.mptab[L], h.faces(L) * sizeof(double)));
    MCK(cudaMemset(h.mptab[L], 0, h.faces(L) * sizeof(double)));
  }
  return ATHG_OK;
}

// The multipole expansion at every level's face positions (after a new expansion)
template <typename T>
int tabulate_multipole(athg_mg* m, Hier<T>& h) {
  if ((int)h.mptab.size() != h.nl) RC(alloc_mptab(h));
  const athg_mg_config& c = m->cfg;
  for (int L = 0; L < h.nl; ++L) {
    k_mp_tab<<<nblk((long long)h.faces(L)), TPB, 0, m->st>>>(
        h.mptab[L], h.n[L], c.x1min, c.x1max, c.x2min, c.x2max, c.x3min, c.x3max, m->mp);
    MCKL();
  }
  return ATHG_OK;
}

// whether the smoothing sweeps of an n^3 level also write its periodic ghost images
// (push_images): every face periodic, n even, and n <= 128. On a GB300 the pushes add
// 0.6-2.3 us to a sweep up to n = 128 against 3.2-3.7 us for a boundary-fill launch, but
// 12.5 us at n = 256 against 6.2 us.
constexpr int kPushMaxN = 128;
bool pushes(const athg_mg* m, int n) {
  return m->periodic && n >= 2 && n % 2 == 0 && n <= kPushMaxN;
}

// whether the two colour sweeps of a smoothing step need a boundary fill between them.
// A ghost next to a non-periodic face (zero gradient, zero-fixed, multipole: a function of
// the interior cell it mirrors) is read only by that cell, which the other colour's sweep
// does not change, so it is filled again before the next sweep of its own colour anyway;
// only periodic ghosts, the images of cells of the other colour, change in between, and
// pushes keep those filled.
bool mid_fill(const athg_mg* m, int n) { return m->any_periodic && !pushes(m, n); }

template <typename T>
int smooth(athg_mg* m, Hier<T>& h, int L, int color, int coff) {
  const int n = h.n[L];
  const double dx = h.dx[L];
  const double isix = 1.15 / 6.0;
  long long nth = (long long)((n + 1) / 2) * n * n;
  if (pushes(m, n))
    k_smooth<T, true><<<nblk(nth), TPB, 0, m->st>>>(h.u[L], h.src[L], n, (T)(dx * dx), (T)isix,
                                                    color ^ coff);
  else
    k_smooth<T, false><<<nblk(nth), TPB, 0, m->st>>>(h.u[L], h.src[L], n, (T)(dx * dx), (T)isix,
                                                     color ^ coff);
  MCKL();
  return ATHG_OK;
}

template <typename T>
int fas_rhs(athg_mg* m, Hier<T>& h, int L) {
  const int n = h.n[L];
  const double dx = h.dx[L];
  k_fas_rhs<T><<<nblk((long long)n * n * n), TPB, 0, m->st>>>(h.u[L], h.src[L], n,
                                                              (T)(1.0 / (dx * dx)));
  MCKL();
  return ATHG_OK;
}

template <typename T>
int store_old(athg_mg* m, Hier<T>& h, int L) {
  MCK(cudaMemcpyAsync(h.uold[L], h.u[L], h.cells(L) * sizeof(T), cudaMemcpyDeviceToDevice, m->st));
  return ATHG_OK;
}


// levels 0..ls of a V-cycle from `top` in one launch (k_vcycle_small)
template <typename T>
int small_vcycle(athg_mg* m, Hier<T>& h, int ls, int top, bool fas, bool homog, bool subtract,
                 int coff) {
  SmallV<T> v{};
  FaceOps f;
  for (int L = 0; L <= ls; ++L) {
    v.u[L] = h.u[L];
    v.src[L] = h.src[L];
    v.uold[L] = fas ? h.uold[L] : nullptr;
    RC(face_ops(m, h, L, homog, &f));
    v.tab[L] = f.tab;
    const double dx = h.dx[L];
    v.dx2[L] = (T)(dx * dx);
    v.idx2[L] = (T)(1.0 / (dx * dx));
  }
  for (int q = 0; q < 6; ++q) v.op[q] = f.op[q];
  v.ls = ls; v.top = top; v.fas = fas ? 1 : 0; v.subtract = subtract ? 1 : 0; v.coff = coff;
  v.push = m->periodic ? 1 : 0;  // pushes(m, 2^L) for every L >= 1 here
  v.anyper = m->any_periodic ? 1 : 0;
  v.isix = (T)(1.15 / 6.0);
  k_vcycle_small<T><<<1, kSmallThreads, small_smem<T>(ls, v.fas), m->st>>>(v);
  MCKL();
  return ATHG_OK;
}

// V(1,1) from level `top` (the current FMG level), multigrid_driver.cpp:684-694
template <typename T>
int vcycle(athg_mg* m, Hier<T>& h, int top, bool fas, bool homog, bool subtract, int& coffset) {
  coffset ^= 1;
  const int coff = coffset;
  // FP32 levels up to n = 16; FP64 ones up to n = 8, since one SM's FP64 rate (1/64 of
  // FP32 on this GPU) makes the 16^3 level faster as separate multi-SM launches
  const int ls = std::min(sizeof(T) == 4 ? kSmallLevels - 1 : kSmallLevels - 2, top);
  // Periodic levels (pushes): the smoothing sweeps keep the ghost layer filled and a level
  // zeroed on the way down has zero ghosts, so the boundary fills left there are the top
  // level's first one and those after prolongation.
  for (int L = top; L > ls; --L) {
    const bool p = pushes(m, h.n[L]);
    if (!p || fas || L == top) RC(apply_bc(m, h, L, homog));
    if (fas && L < top) { RC(store_old(m, h, L)); RC(fas_rhs(m, h, L)); }
    RC(smooth(m, h, L, 0, coff));
    if (mid_fill(m, h.n[L])) RC(apply_bc(m, h, L, homog));
    RC(smooth(m, h, L, 1, coff));
    if (!p) RC(apply_bc(m, h, L, homog));
    const int nc = h.n[L - 1];
    const double dx = h.dx[L];
    k_defect_restrict<T><<<nblk((long long)nc * nc * nc), TPB, 0, m->st>>>(
        h.u[L], h.src[L], h.src[L - 1], h.u[L - 1], nc, (T)(1.0 / (dx * dx)), fas ? 1 : 0);
    MCKL();
    if (!fas) MCK(cudaMemsetAsync(h.u[L - 1], 0, h.cells(L - 1) * sizeof(T), m->st));
  }
  RC(small_vcycle(m, h, ls, top, fas, homog, subtract, coff));
  for (int L = ls; L < top; ++L) {
    // the one-block levels' last sweep pushed too when pushes(): n = 2^ls <= 16
    if (!pushes(m, h.n[L])) RC(apply_bc(m, h, L, homog));
    const int nc = h.n[L];
    k_prolong_correct<T><<<nblk((long long)nc * nc * nc), TPB, 0, m->st>>>(
        h.u[L], fas ? h.uold[L] : nullptr, h.u[L + 1], nc);
    MCKL();
    RC(apply_bc(m, h, L + 1, homog));
    RC(smooth(m, h, L + 1, 0, coff));
    if (mid_fill(m, h.n[L + 1])) RC(apply_bc(m, h, L + 1, homog));
    RC(smooth(m, h, L + 1, 1, coff));
  }
  // the ghost layer of the result (callers read it: FMG prolongation, the next cycle)
  if (!pushes(m, h.n[top])) RC(apply_bc(m, h, top, homog));
  return ATHG_OK;
}

// the mean of level L's interior into m->red[1] (the sum in m->red[0]): total = sum * dx^3
// (Multigrid::CalculateTotal), average = total / volume
template <typename T>
int level_mean(athg_mg* m, Hier<T>& h, const T* a, int L) {
  const int n = h.n[L];
  MCK(cudaMemsetAsync(m->red, 0, sizeof(double), m->st));
  k_sum<T><<<nblk((long long)n * n * col_chunks(n)), TPB, 0, m->st>>>(a, n, m->red);
  MCKL();
  const double dxl = h.dx[L];
  k_mean<<<1, 1, 0, m->st>>>(m->red, dxl * dxl * dxl / m->vol);
  MCKL();
  return ATHG_OK;
}

template <typename T>
int subtract_mean(athg_mg* m, Hier<T>& h, T* a, int L) {
  RC(level_mean(m, h, a, L));
  k_sub_const<T><<<nblk((long long)h.cells(L)), TPB, 0, m->st>>>(a, (long long)h.cells(L),
                                                                m->red + 1);
  MCKL();
  return ATHG_OK;
}

// FMG: source restriction through all levels, then V(1,1) at each level followed by
// FMG prolongation (MultigridDriver::SolveFMGCycle)
template <typename T>
int fmg(athg_mg* m, Hier<T>& h, bool fas, bool subtract, int& coffset) {
  const int top = h.nl - 1;
  for (int L = top; L > 0; --L) {
    const int nc = h.n[L - 1];
    k_restrict<T><<<nblk((long long)nc * nc * nc), TPB, 0, m->st>>>(h.src[L], h.src[L - 1], nc);
    MCKL();
  }
  for (int f = 0; f <= top; ++f) {
    // vcycle() leaves level f's ghost layer filled for the FMG prolongation
    RC(vcycle(m, h, f, fas, false, subtract, coffset));
    if (f != top) {
      const int nc = h.n[f];
      k_fmg_prolong<T><<<nblk((long long)nc * nc * nc), TPB, 0, m->st>>>(h.u[f], h.u[f + 1], nc);
      MCKL();
    }
  }
  return ATHG_OK;
}

int defect_norm64(athg_mg* m, double* out) {
  Hier<double>& h = m->h64;
  const int L = h.nl - 1, n = h.n[L];
  RC(apply_bc(m, h, L, false));
  MCK(cudaMemsetAsync(m->red, 0, sizeof(double), m->st));
  const double dx = h.dx[L];
  const double idx2 = 1.0 / (dx * dx);
  const float idx2_hi = (float)idx2, idx2_lo = (float)(idx2 - (double)idx2_hi);
  k_defect_sq<<<nblk((long long)n * n * col_chunks(n)), TPB, 0, m->st>>>(
      h.u[L], h.src[L], n, idx2, idx2_hi, idx2_lo, m->cfg.precision == ATHG_MIXED ? 1 : 0,
      m->red);
  MCKL();
  double s;
  MCK(cudaMemcpyAsync(&s, m->red, sizeof(double), cudaMemcpyDeviceToHost, m->st));
  MCK(cudaStreamSynchronize(m->st));
  // multigrid.cpp:594 (sum * dV), multigrid_driver.cpp:849-856 (/ volume, sqrt)
  *out = std::sqrt(s * dx * dx * dx / m->vol);
  return ATHG_OK;
}

int multipole_setup(athg_mg* m) {
  Hier<double>& h = m->h64;
  const int L = h.nl - 1, n = h.n[L];
  const athg_mg_config& c = m->cfg;
  // cell volume from the level's face positions (multigrid.cpp:1063-1064)
  auto xf = [&](int i, double lo, double hi) {
    return i == 1 ? lo : (i == n + 1 ? hi : lo + (i - 1) * ((hi - lo) / n));
  };
  double vol = (xf(2, c.x1min, c.x1max) - xf(1, c.x1min, c.x1max)) *
               (xf(2, c.x2min, c.x2max) - xf(1, c.x2min, c.x2max)) *
               (xf(2, c.x3min, c.x3max) - xf(1, c.x3min, c.x3max));
  double origin[3] = {c.mporigin[0], c.mporigin[1], c.mporigin[2]};
  if (c.auto_mporigin) {
    MCK(cudaMemsetAsync(m->red, 0, 4 * sizeof(double), m->st));
    k_com<<<nblk((long long)n * n * col_chunks(n)), TPB, 0, m->st>>>(
        h.src[L], n, c.x1min, c.x1max, c.x2min, c.x2max, c.x3min, c.x3max, vol, m->red);
    MCKL();
    double s[4];
    MCK(cudaMemcpyAsync(s, m->red, sizeof(s), cudaMemcpyDeviceToHost, m->st));
    MCK(cudaStreamSynchronize(m->st));
    double im = 1.0 / s[0];
    origin[0] = im * s[3]; origin[1] = im * s[1]; origin[2] = im * s[2];
  }
  MCK(cudaMemcpyAsync(m->mpo_d, origin, sizeof(origin), cudaMemcpyHostToDevice, m->st));
  MCK(cudaMemsetAsync(m->red, 0, 25 * sizeof(double), m->st));
  k_moments<<<nblk((long long)n * n * col_chunks(n)), TPB, 0, m->st>>>(
      h.src[L], n, c.x1min, c.x1max, c.x2min, c.x2max, c.x3min, c.x3max, vol, m->mpo_d,
      c.mporder, c.nodipole, m->red);
  MCKL();
  double mm[25];
  MCK(cudaMemcpyAsync(mm, m->red, sizeof(mm), cudaMemcpyDeviceToHost, m->st));
  MCK(cudaStreamSynchronize(m->st));
  const double PI = 3.1415926535897932;
  const double c0 = -0.25 / PI, c1 = -0.25 / PI, c2 = -0.0625 / PI, c2a = -0.75 / PI;
  const double c30 = -0.0625 / PI, c31 = -0.0625 * 1.5 / PI, c32 = -0.25 * 15.0 / PI,
               c33 = -0.0625 * 2.5 / PI;
  const double c40 = -0.0625 * 0.0625 / PI, c41 = -0.0625 * 2.5 / PI, c42 = -0.0625 * 5.0 / PI,
               c43 = -0.0625 * 17.5 / PI, c44 = -0.25 * 35.0 / PI;
  const double sc[25] = {c0, c1, c1, c1, c2a, c2a, c2, c2a, c2a, c33, c32, c31, c30,
                         c31, c32, c33, c44, c43, c42, c41, c40, c41, c42, c43, c44};
  const int nc = c.mporder == 4 ? 25 : 9;
  for (int q = 0; q < 25; ++q) m->mp.c[q] = q < nc ? mm[q] * sc[q] : 0.0;
  for (int d = 0; d < 3; ++d) m->mp.o[d] = origin[d];
  m->mp.order = c.mporder;
  RC(tabulate_multipole(m, m->h64));
  if (m->cfg.precision == ATHG_MIXED) RC(tabulate_multipole(m, m->h32));
  return ATHG_OK;
}

// mixed path: FP32 V-cycle on the correction equation for the current FP64 defect,
// correction accumulated into the FP64 solution
int refine_once(athg_mg* m) {
  Hier<double>& H = m->h64;
  Hier<float>& h = m->h32;
  const int top = h.nl - 1, n = h.n[top];
  RC(apply_bc(m, H, top, false));
  const double dx = H.dx[top];
  const double idx2 = 1.0 / (dx * dx);
  const float idx2_hi = (float)idx2, idx2_lo = (float)(idx2 - (double)idx2_hi);
  k_defect_to32<<<nblk((long long)n * n * n), TPB, 0, m->st>>>(H.u[top], H.src[top], n, idx2,
                                                               idx2_hi, idx2_lo, h.src[top]);
  MCKL();
  MCK(cudaMemsetAsync(h.u[top], 0, h.cells(top) * sizeof(float), m->st));
  RC(vcycle(m, h, top, false, true, m->subtract, m->coffset32));
  k_add_correction<<<nblk((long long)h.cells(top)), TPB, 0, m->st>>>(H.u[top], h.u[top],
                                                                     (long long)h.cells(top));
  MCKL();
  return ATHG_OK;
}

int one_cycle(athg_mg* m) {
  const int top = m->lmax;
  if (m->cfg.precision == ATHG_MIXED) return refine_once(m);
  return vcycle(m, m->h64, top, m->fas, false, m->subtract, m->coffset);
}

// one_cycle from a captured CUDA graph: the ~20-200 small launches of a V-cycle become one
// graph launch. Not used while the stream is itself being captured (the self-gravity
// solve inside a captured hydro cycle).
int cycle(athg_mg* m) {
  cudaStreamCaptureStatus cs = cudaStreamCaptureStatusNone;
  MCK(cudaStreamIsCapturing(m->st, &cs));
  if (cs != cudaStreamCaptureStatusNone) return one_cycle(m);
  const bool mixed = m->cfg.precision == ATHG_MIXED;
  int& coff = mixed ? m->coffset32 : m->coffset;
  const int par = coff & 1;
  if (!m->cyc_exec[par]) {
    const int c32 = m->coffset32, c64 = m->coffset;
    MCK(cudaStreamBeginCapture(m->st, cudaStreamCaptureModeThreadLocal));
    int rc = one_cycle(m);
    cudaGraph_t gr = nullptr;
    cudaError_t e = cudaStreamEndCapture(m->st, &gr);
    m->coffset32 = c32;
    m->coffset = c64;
    if (rc) {
      if (gr) cudaGraphDestroy(gr);
      return rc;
    }
    if (e != cudaSuccess) return mgfail(ATHG_ERR_CUDA, "multigrid cycle capture failed");
    m->cyc_graph[par] = gr;
    MCK(cudaGraphInstantiate(&m->cyc_exec[par], gr, 0));
  }
  MCK(cudaGraphLaunch(m->cyc_exec[par], m->st));
  coff ^= 1;  // what the captured cycle did to the host-side colour offset
  return ATHG_OK;
}

}  // namespace

extern "C" {

int athg_mg_create(const athg_mg_config* cfg, athg_mg** out) {
  if (!cfg || !out) return mgfail(ATHG_ERR_ARG, "null argument");
  *out = nullptr;
  int n = cfg->nx, lmax = 0;
  if (n < 2 || (n & (n - 1)) != 0) return mgfail(ATHG_ERR_ARG, "nx must be a power of two >= 2");
  if (n > 4096) return mgfail(ATHG_ERR_ARG, "nx too large");
  while ((1 << lmax) < n) ++lmax;
  for (int f = 0; f < 6; ++f)
    if (cfg->bc[f] < ATHG_MG_PERIODIC || cfg->bc[f] > ATHG_MG_MULTIPOLE)
      return mgfail(ATHG_ERR_ARG, "unknown multigrid boundary type");
  for (int d = 0; d < 3; ++d)
    if ((cfg->bc[2 * d] == ATHG_MG_PERIODIC) != (cfg->bc[2 * d + 1] == ATHG_MG_PERIODIC))
      return mgfail(ATHG_ERR_ARG, "periodic boundaries must be set on both faces of an axis");
  if (cfg->precision != ATHG_FP64 && cfg->precision != ATHG_MIXED)
    return mgfail(ATHG_ERR_ARG, "precision must be ATHG_FP64 or ATHG_MIXED");
  if (cfg->threshold < 0.0 && cfg->niteration < 0)
    return mgfail(ATHG_ERR_ARG, "set a threshold >= 0 or niteration >= 0");
  int ndev = 0;
  if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev == 0)
    return mgfail(ATHG_ERR_CUDA, "no CUDA device available");
  athg_mg* m = new athg_mg();
  m->cfg = *cfg;
  m->lmax = lmax;
  for (int f = 0; f < 6; ++f) {
    if (cfg->bc[f] != ATHG_MG_PERIODIC) m->periodic = false;
    else m->any_periodic = true;
    if (cfg->bc[f] == ATHG_MG_MULTIPOLE) m->any_mp = true;
  }
  if (m->any_mp && cfg->mporder != 2 && cfg->mporder != 4) {
    delete m;
    return mgfail(ATHG_ERR_ARG, "mporder must be 2 or 4 with multipole boundaries");
  }
  // multigrid_driver.cpp:139-300: the mean source is removed unless a face is multipole,
  // which switches on the full approximation scheme instead
  m->subtract = !m->any_mp;
  m->fas = m->any_mp;
  m->rdx = (cfg->x1max - cfg->x1min) / (double)n;
  m->vol = (cfg->x1max - cfg->x1min) * (cfg->x2max - cfg->x2min) * (cfg->x3max - cfg->x3min);
  int rc;
  if (cudaStreamCreateWithFlags(&m->st, cudaStreamNonBlocking) != cudaSuccess) {
    delete m;
    return mgfail(ATHG_ERR_CUDA, "cudaStreamCreate failed");
  }
  m->own_st = m->st;
  if (cfg->precision == ATHG_MIXED) {
    // FP64 solution and source on the finest level only; FP32 hierarchy for the cycles
    rc = alloc_top(m->h64, lmax, m->rdx);
    if (!rc) rc = alloc_hier(m->h32, lmax, m->rdx, m->fas);
  } else {
    rc = alloc_hier(m->h64, lmax, m->rdx, m->fas);
  }
  if (!rc && cudaMalloc(&m->red, 32 * sizeof(double)) != cudaSuccess) rc = ATHG_ERR_CUDA;
  if (!rc && cudaMalloc(&m->mpo_d, 4 * sizeof(double)) != cudaSuccess) rc = ATHG_ERR_CUDA;
  // shared memory of the coarse-level kernel (levels up to n = 16, three arrays each)
  if (!rc && (cudaFuncSetAttribute(k_vcycle_small<double>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                   (int)small_smem<double>(kSmallLevels - 1, 1)) != cudaSuccess ||
              cudaFuncSetAttribute(k_vcycle_small<float>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                   (int)small_smem<float>(kSmallLevels - 1, 1)) != cudaSuccess))
    rc = ATHG_ERR_CUDA;
  // multipole faces before the first expansion: phi = 0 on every face
  if (!rc && m->any_mp) rc = alloc_mptab(m->h64);
  if (!rc && m->any_mp && cfg->precision == ATHG_MIXED) rc = alloc_mptab(m->h32);
  if (rc) {
    athg_mg_destroy(m);
    return mgfail(ATHG_ERR_CUDA, "multigrid allocation failed");
  }
  *out = m;
  return ATHG_OK;
}

int athg_mg_destroy(athg_mg* m) {
  if (!m) return ATHG_OK;
  free_hier(m->h64);
  free_hier(m->h32);
  if (m->red) cudaFree(m->red);
  if (m->mpo_d) cudaFree(m->mpo_d);
  for (int q = 0; q < 2; ++q) {
    if (m->cyc_exec[q]) cudaGraphExecDestroy(m->cyc_exec[q]);
    if (m->cyc_graph[q]) cudaGraphDestroy(m->cyc_graph[q]);
  }
  if (m->own_st) cudaStreamDestroy(m->own_st);
  delete m;
  return ATHG_OK;
}

int athg_mg_load_source(athg_mg* m, const double* rho, size_t count, double fac) {
  if (!m || !rho) return mgfail(ATHG_ERR_ARG, "null argument");
  const int n = 1 << m->lmax, nt = n + 2;
  if (count != (size_t)n * n * n) return mgfail(ATHG_ERR_ARG, "source size mismatch");
  std::vector<double> full((size_t)nt * nt * nt, 0.0);
  for (int k = 0; k < n; ++k)
    for (int j = 0; j < n; ++j)
      for (int i = 0; i < n; ++i)
        full[ix(nt, k + 1, j + 1, i + 1)] =
            (fac == 1.0) ? rho[((size_t)k * n + j) * n + i] : rho[((size_t)k * n + j) * n + i] * fac;
  MCK(cudaMemcpyAsync(m->h64.src[m->lmax], full.data(), full.size() * 8, cudaMemcpyHostToDevice,
                      m->st));
  MCK(cudaStreamSynchronize(m->st));
  return ATHG_OK;
}

int athg_mg_set_phi(athg_mg* m, const double* phi, size_t count) {
  if (!m || !phi) return mgfail(ATHG_ERR_ARG, "null argument");
  const int n = 1 << m->lmax, nt = n + 2;
  if (count != (size_t)n * n * n) return mgfail(ATHG_ERR_ARG, "phi size mismatch");
  std::vector<double> full((size_t)nt * nt * nt, 0.0);
  for (int k = 0; k < n; ++k)
    for (int j = 0; j < n; ++j)
      for (int i = 0; i < n; ++i) full[ix(nt, k + 1, j + 1, i + 1)] = phi[((size_t)k * n + j) * n + i];
  MCK(cudaMemcpyAsync(m->h64.u[m->lmax], full.data(), full.size() * 8, cudaMemcpyHostToDevice,
                      m->st));
  MCK(cudaStreamSynchronize(m->st));
  return ATHG_OK;
}

int athg_mg_get_phi(athg_mg* m, double* phi, size_t count) {
  if (!m || !phi) return mgfail(ATHG_ERR_ARG, "null argument");
  const int n = 1 << m->lmax, nt = n + 2;
  if (count != (size_t)n * n * n) return mgfail(ATHG_ERR_ARG, "phi size mismatch");
  std::vector<double> full((size_t)nt * nt * nt);
  MCK(cudaMemcpyAsync(full.data(), m->h64.u[m->lmax], full.size() * 8, cudaMemcpyDeviceToHost,
                      m->st));
  MCK(cudaStreamSynchronize(m->st));
  for (int k = 0; k < n; ++k)
    for (int j = 0; j < n; ++j)
      for (int i = 0; i < n; ++i) phi[((size_t)k * n + j) * n + i] = full[ix(nt, k + 1, j + 1, i + 1)];
  return ATHG_OK;
}

}  // extern "C"

namespace athg {

int mg_finest(athg_mg* m, double** u, double** src, int* n) {
  if (!m) return mgfail(ATHG_ERR_ARG, "null multigrid");
  *u = m->h64.u[m->lmax];
  *src = m->h64.src[m->lmax];
  *n = 1 << m->lmax;
  return ATHG_OK;
}

int mg_bind_stream(athg_mg* m, cudaStream_t st) {
  if (!m) return mgfail(ATHG_ERR_ARG, "null multigrid");
  m->st = st ? st : m->own_st;
  return ATHG_OK;
}

bool mg_solve_capturable(const athg_mg* m) {
  return m && m->cfg.threshold < 0.0 && !m->any_mp;
}

int mg_solve(athg_mg* m, bool want_norm, int* iterations, double* defect_norm) {
  const int top = m->lmax;
  Hier<double>& H = m->h64;
  m->iterations = 0;
  // mixed FMG: the mean subtractions of the source and of the FMG solution ride on the
  // narrowing and widening passes (k_sub_narrow, k_widen_sub)
  const bool mixed_fmg = m->cfg.mode == ATHG_MG_FMG && m->cfg.precision == ATHG_MIXED;
  if (m->subtract) {
    if (mixed_fmg) RC(level_mean(m, H, H.src[top], top));
    else RC(subtract_mean(m, H, H.src[top], top));
  }
  if (m->any_mp) RC(multipole_setup(m));
  if (m->cfg.mode == ATHG_MG_FMG) {
    if (mixed_fmg) {
      Hier<float>& h = m->h32;
      const long long c = (long long)h.cells(top);
      if (m->subtract) {
        k_sub_narrow<<<nblk(c), TPB, 0, m->st>>>(H.src[top], h.src[top], c, m->red + 1);
      } else {
        k_narrow<<<nblk(c), TPB, 0, m->st>>>(H.src[top], h.src[top], c);
      }
      MCKL();
      RC(fmg(m, h, m->fas, m->subtract, m->coffset32));
      if (m->subtract) {
        RC(level_mean(m, h, h.u[top], top));
        k_widen_sub<<<nblk(c), TPB, 0, m->st>>>(h.u[top], H.u[top], c, m->red + 1);
      } else {
        k_widen<<<nblk(c), TPB, 0, m->st>>>(h.u[top], H.u[top], c);
      }
      MCKL();
    } else {
      RC(fmg(m, H, m->fas, m->subtract, m->coffset));
      if (m->subtract) RC(subtract_mean(m, H, H.u[top], top));
    }
  }
  double def = 0.0;
  if (m->cfg.threshold >= 0.0) {  // SolveIterative (multigrid_driver.cpp:721-760)
    RC(defect_norm64(m, &def));
    int nit = 0;
    while (def > m->cfg.threshold) {
      RC(cycle(m));
      m->iterations++;
      double old = def;
      RC(defect_norm64(m, &def));
      if (def / old > 0.8 && m->cfg.threshold == 0.0) break;
      if (nit > 100) break;
      nit++;
    }
  } else {
    for (int q = 0; q < m->cfg.niteration; ++q) {
      RC(cycle(m));
      m->iterations++;
    }
    if (want_norm) RC(defect_norm64(m, &def));
  }
  if (m->subtract) RC(subtract_mean(m, H, H.u[top], top));
  RC(apply_bc(m, H, top, false));
  if (want_norm) MCK(cudaStreamSynchronize(m->st));
  m->last_norm = def;
  if (iterations) *iterations = m->iterations;
  if (defect_norm) *defect_norm = def;
  return ATHG_OK;
}

}  // namespace athg

extern "C" {

int athg_mg_solve(athg_mg* m, int* iterations, double* defect_norm) {
  if (!m) return mgfail(ATHG_ERR_ARG, "null argument");
  return athg::mg_solve(m, true, iterations, defect_norm);
}

int athg_mg_vcycles(athg_mg* m, int n) {
  if (!m) return mgfail(ATHG_ERR_ARG, "null argument");
  for (int q = 0; q < n; ++q) RC(cycle(m));
  return ATHG_OK;
}

int athg_mg_defect_norm(athg_mg* m, double* out) {
  if (!m || !out) return mgfail(ATHG_ERR_ARG, "null argument");
  return defect_norm64(m, out);
}

int athg_mg_stream(athg_mg* m, void** stream) {
  if (!m || !stream) return mgfail(ATHG_ERR_ARG, "null argument");
  *stream = (void*)m->st;
  return ATHG_OK;
}

int athg_mg_multipole(athg_mg* m, double* out28) {
  if (!m || !out28) return mgfail(ATHG_ERR_ARG, "null argument");
  for (int q = 0; q < 25; ++q) out28[q] = m->mp.c[q];
  for (int d = 0; d < 3; ++d) out28[25 + d] = m->mp.o[d];
  return ATHG_OK;
}

}  // extern "C"
