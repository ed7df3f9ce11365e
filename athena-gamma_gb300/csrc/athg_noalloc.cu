// athg_noalloc.cu -- CFL time step of one caller-owned MeshBlock without any device
// allocation (athg_block_cfl_dt_noalloc, declared in include/athena_gb300.h).
//
// Some callers cannot allocate device memory: code that must not synchronise the device
// (cudaMalloc and cudaFree may), hosts whose device memory is handed out by their own pool
// and must not be touched by a library, or drivers with a fixed memory budget set up
// before the run. This entry point computes the same minimum as athg_new_block_dt (the
// reference's Hydro::NewBlockTimeStep for one block), but takes the block's arrays from
// the caller and keeps its scratch -- one partial minimum per thread block -- in a
// file-scope device array of fixed size instead of memory from cudaMalloc.
//
// The scratch array lives in every GPU that loads this library until the process exits
// (kMaxPartials doubles). All calls share it and it keeps the last call's contents:
// every call writes each partial it later reads, so nothing has to start at zero, but two
// calls that overlap on the GPU (for example on two streams) race on it.
#include <cstring>
#include <string>

#include "athena_gb300.h"
#include "athg_device.cuh"

namespace athg {
void set_last_error(const std::string& s);
}

namespace {

using namespace athg;

constexpr int kThreads = 256;
constexpr int kCellsPerThread = 8;
// partial minima the scratch array holds: with kThreads * kCellsPerThread cells per
// thread block this covers blocks of up to 8192 * 2048 = 16,777,216 interior cells
constexpr int kMaxPartials = 8192;

static __device__ __align__(256) double g_dt_partials[kMaxPartials];


int fail(int code, const std::string& msg) {
  set_last_error(msg);
  return code;
}

struct BlockArgs {
  const double *w, *bcc, *b1, *b2, *b3;
  int nx1, nx2, nx3, ng, nc1, nc2, mhd;
  double gamma, dx1, dx2, dx3;
  long long ncell, nf1, nf2;
};

__device__ inline long long cell(const BlockArgs& a, int k, int j, int i) {
  return ((long long)k * a.nc2 + j) * a.nc1 + i;
}

// pass 1: each thread block reduces up to kThreads*kCellsPerThread interior cells and
// writes one partial minimum (same per-cell formula as the pool kernel k_block_dt)
__global__ void __launch_bounds__(kThreads) k_dt_partials(BlockArgs a, double* partials) {
  const long long ncells = (long long)a.nx1 * a.nx2 * a.nx3;
  const long long base = (long long)blockIdx.x * kThreads * kCellsPerThread;
  double mindt = 1.79769313486231570815e308;
  for (int r = 0; r < kCellsPerThread; ++r) {
    long long t = base + (long long)r * kThreads + threadIdx.x;
    if (t >= ncells) break;
    int i = (int)(t % a.nx1) + a.ng;
    long long q = t / a.nx1;
    int j = (int)(q % a.nx2) + a.ng, k = (int)(q / a.nx2) + a.ng;
    const long long c = cell(a, k, j, i), nc = a.ncell;
    double d = a.w[c], vx = a.w[nc + c], vy = a.w[2 * nc + c], vz = a.w[3 * nc + c];
    double pr = a.w[4 * nc + c];
    double dt1, dt2, dt3;
    if (a.mhd) {
      double bc1 = a.bcc[c], bc2 = a.bcc[nc + c], bc3 = a.bcc[2 * nc + c];
      long long f1 = ((long long)k * a.nc2 + j) * (a.nc1 + 1) + i;
      long long f2 = ((long long)k * (a.nc2 + 1) + j) * a.nc1 + i;
      double bx1 = bc1 + fabs(a.b1[f1] - bc1);
      double cf = fast_speed<double>(d, pr, bc2, bc3, bx1, a.gamma);
      dt1 = a.dx1 / (fabs(vx) + cf);
      double bx2 = bc2 + fabs(a.b2[f2] - bc2);
      cf = fast_speed<double>(d, pr, bc3, bc1, bx2, a.gamma);
      dt2 = a.dx2 / (fabs(vy) + cf);
      double bx3 = bc3 + fabs(a.b3[c] - bc3);
      cf = fast_speed<double>(d, pr, bc1, bc2, bx3, a.gamma);
      dt3 = a.dx3 / (fabs(vz) + cf);
    } else {
      double cs = sqrt(a.gamma * pr / d);
      dt1 = a.dx1 / (fabs(vx) + cs);
      dt2 = a.dx2 / (fabs(vy) + cs);
      dt3 = a.dx3 / (fabs(vz) + cs);
    }
    mindt = mn(mn(mn(mindt, dt1), dt2), dt3);
  }
  for (int o = 16; o > 0; o >>= 1) mindt = mn(mindt, __shfl_xor_sync(0xffffffffu, mindt, o));
  __shared__ double red[kThreads / 32];
  if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = mindt;
  __syncthreads();
  if (threadIdx.x < 32) {
    double v = threadIdx.x < kThreads / 32 ? red[threadIdx.x] : 1.79769313486231570815e308;
    for (int o = 16; o > 0; o >>= 1) v = mn(v, __shfl_xor_sync(0xffffffffu, v, o));
    if (threadIdx.x == 0) partials[blockIdx.x] = v;
  }
}

// pass 2: one thread block folds the partials and applies the CFL number
__global__ void __launch_bounds__(kThreads)
k_dt_final(const double* partials, int n, double cfl, double* out) {
  double v = 1.79769313486231570815e308;
  for (int t = threadIdx.x; t < n; t += kThreads) v = mn(v, partials[t]);
  for (int o = 16; o > 0; o >>= 1) v = mn(v, __shfl_xor_sync(0xffffffffu, v, o));
  __shared__ double red[kThreads / 32];
  if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = v;
  __syncthreads();
  if (threadIdx.x < 32) {
    double r = threadIdx.x < kThreads / 32 ? red[threadIdx.x] : 1.79769313486231570815e308;
    for (int o = 16; o > 0; o >>= 1) r = mn(r, __shfl_xor_sync(0xffffffffu, r, o));
    if (threadIdx.x == 0) *out = r * cfl;
  }
}

}  // namespace

extern "C" int athg_block_cfl_dt_noalloc(const athg_config* cfg, const double* w,
                                         const double* bcc, const double* b1f,
                                         const double* b2f, const double* b3f, double dx1,
                                         double dx2, double dx3, double* dt_out,
                                         void* stream) {
  if (!cfg || !w || !dt_out) return fail(ATHG_ERR_ARG, "null argument");
  if (cfg->magnetic && (!bcc || !b1f || !b2f || !b3f))
    return fail(ATHG_ERR_ARG, "MHD needs bcc and the three face fields");
  if (cfg->nx1 < 1 || cfg->nx2 < 1 || cfg->nx3 < 1 || cfg->nghost < 0)
    return fail(ATHG_ERR_ARG, "bad block size");
  const long long ncells = (long long)cfg->nx1 * cfg->nx2 * cfg->nx3;
  const long long per_block = (long long)kThreads * kCellsPerThread;
  const long long nparts = (ncells + per_block - 1) / per_block;
  if (nparts > kMaxPartials)
    return fail(ATHG_ERR_ARG,
                "block too large for athg_block_cfl_dt_noalloc: " + std::to_string(ncells) +
                    " interior cells, at most " + std::to_string((long long)kMaxPartials * per_block));
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess) return fail(ATHG_ERR_CUDA, "no current CUDA device");
  // the scratch array's address in the current device's context, looked up on every call
  // (a host-side lookup, no allocation): a cached address would go stale when the context
  // is replaced (cudaDeviceReset), and nothing is shared between host threads. The first
  // call on a device loads this library's device code there.
  double* partials = nullptr;
  {
    cudaError_t e = cudaGetSymbolAddress((void**)&partials, g_dt_partials);
    if (e != cudaSuccess)
      return fail(ATHG_ERR_CUDA, std::string("cudaGetSymbolAddress: ") + cudaGetErrorString(e));
  }
  BlockArgs a;
  a.w = w; a.bcc = bcc; a.b1 = b1f; a.b2 = b2f; a.b3 = b3f;
  a.nx1 = cfg->nx1; a.nx2 = cfg->nx2; a.nx3 = cfg->nx3; a.ng = cfg->nghost;
  a.nc1 = cfg->nx1 + 2 * cfg->nghost; a.nc2 = cfg->nx2 + 2 * cfg->nghost;
  const int nc3 = cfg->nx3 + 2 * cfg->nghost;
  a.ncell = (long long)a.nc1 * a.nc2 * nc3;
  a.nf1 = (long long)nc3 * a.nc2 * (a.nc1 + 1);
  a.nf2 = (long long)nc3 * (a.nc2 + 1) * a.nc1;
  a.mhd = cfg->magnetic ? 1 : 0;
  a.gamma = cfg->gamma;
  a.dx1 = dx1; a.dx2 = dx2; a.dx3 = dx3;
  cudaStream_t st = (cudaStream_t)stream;
  k_dt_partials<<<(unsigned)nparts, kThreads, 0, st>>>(a, partials);
  k_dt_final<<<1, kThreads, 0, st>>>(partials, (int)nparts, cfg->cfl_number, dt_out);
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess)
    return fail(ATHG_ERR_CUDA, std::string("kernel launch: ") + cudaGetErrorString(e));
  return ATHG_OK;
}
