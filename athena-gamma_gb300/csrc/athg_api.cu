// athg_api.cu -- the C ABI: context, device block pool, stage sequencing and the
// CUDA-graph cycle. Declarations and reference interfaces: include/athena_gb300.h.
#include <algorithm>
#include <cmath>
#include <set>
#include <tuple>
#include <type_traits>
#include <utility>
#include <cstdio>
#include <cstring>
#include <string>
#include <vector>

#include "athena_gb300.h"
#include "athg_bvals.cuh"
#include "athg_launch.cuh"
#include "athg_amr.h"
#include "athg_single_pass.h"
#include "athg_df.h"
#include "athg_fft.h"
#include "athg_internal.h"

using namespace athg;

namespace {
thread_local std::string g_err;

int fail(int code, const std::string& msg) {
  g_err = msg;
  return code;
}

#define CK(call)                                                                        \
  do {                                                                                  \
    cudaError_t e_ = (call);                                                            \
    if (e_ != cudaSuccess)                                                              \
      return fail(ATHG_ERR_CUDA, std::string(#call) + ": " + cudaGetErrorString(e_));  \
  } while (0)

#define CKL()                                                                           \
  do {                                                                                  \
    cudaError_t e_ = cudaGetLastError();                                                \
    if (e_ != cudaSuccess)                                                              \
      return fail(ATHG_ERR_CUDA, std::string("kernel launch: ") + cudaGetErrorString(e_)); \
  } while (0)

constexpr double kDblMax = 1.79769313486231570815e308;

// time += dt, ncycle++ (when advancing), then Mesh::NewTimeStep
// (reference src/mesh/mesh.cpp:1078-1118). The block minimum is read and reset.
__global__ void k_end_cycle(double* time, double* dt, long long* ncycle,
                            unsigned long long* dtmin, double cfl, double tlim, int advance,
                            float* dtf, unsigned int* err) {
  if (threadIdx.x != 0 || blockIdx.x != 0) return;
  double t = *time, d = *dt;
  if (advance) {
    t += d;
    *ncycle += 1;
  }
  double bdt = __longlong_as_double((long long)*dtmin) * cfl;
  d = 2.0 * d;
  d = (bdt < d) ? bdt : d;
  if (t < tlim && (tlim - t) < d) d = tlim - t;
  // device error word, bit 1: a time step that is not a positive finite number
  if (!(d > 0.0 && d <= 1.79769313486231570815e308)) atomicOr(err, kErrTimeStep);
  *time = t;
  *dt = d;
  if (dtf) *dtf = (float)d;  // the flux kernels of the mixed path read dt in FP32
  *dtmin = (unsigned long long)__double_as_longlong(kDblMax);
}

// max |div B| * dx over interior cells (the quantity CT keeps at round-off)
__global__ void k_divb(Geom g, const double* b1, const double* b2, const double* b3,
                       const BlockGeo* geo, unsigned long long* out) {
  const int t = blockIdx.x * blockDim.x + threadIdx.x;
  double v = 0.0;
  if (t < g.nx1 * g.nx2) {
    const int jj = t / g.nx1, i = g.is + t - jj * g.nx1, j = g.js + jj;
    const int k = g.ks + blockIdx.y, b = blockIdx.z;
    const double* p1 = b1 + (int64_t)b * g.nf1;
    const double* p2 = b2 + (int64_t)b * g.nf2;
    const double* p3 = b3 + (int64_t)b * g.nf3;
    const BlockGeo ge = geo[b];
    double d = (p1[f1idx(g, k, j, i + 1)] - p1[f1idx(g, k, j, i)]) / ge.dx[0] +
               (p2[f2idx(g, k, j + 1, i)] - p2[f2idx(g, k, j, i)]) / ge.dx[1] +
               (p3[f3idx(g, k + 1, j, i)] - p3[f3idx(g, k, j, i)]) / ge.dx[2];
    double h = fmin(ge.dx[0], fmin(ge.dx[1], ge.dx[2]));
    v = fabs(d) * h;
  }
  for (int o = 16; o > 0; o >>= 1) v = fmax(v, __shfl_xor_sync(0xffffffffu, v, o));
  if ((threadIdx.x & 31) == 0) atomicMax(out, (unsigned long long)__double_as_longlong(v));
}

// volume integral of the conserved variables (history output, src/outputs/history.cpp)
__global__ void k_sum_cons(Geom g, const double* u, const BlockGeo* geo, double* out) {
  const int t = blockIdx.x * blockDim.x + threadIdx.x;
  double s[5] = {0, 0, 0, 0, 0};
  if (t < g.nx1 * g.nx2) {
    const int jj = t / g.nx1, i = g.is + t - jj * g.nx1, j = g.js + jj;
    const int k = g.ks + blockIdx.y, b = blockIdx.z;
    const BlockGeo ge = geo[b];
    const double vol = ge.dx[0] * ge.dx[1] * ge.dx[2];
    const double* ub = u + (int64_t)b * NHYD * g.ncell;
    for (int n = 0; n < 5; ++n) s[n] = ub[n * g.ncell + cidx(g, k, j, i)] * vol;
  }
  for (int n = 0; n < 5; ++n) {
    double v = s[n];
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    if ((threadIdx.x & 31) == 0) atomicAdd(out + n, v);
  }
}

// HistoryOutput::WriteOutputFile sums (outputs/history.cpp:45-130): volume-weighted mass,
// momenta, kinetic energy per direction, total energy, 1/2 rho phi (with self-gravity)
// and magnetic energy per direction, over interior cells. One partial per thread block
// (warp shuffles, then shared memory), summed on the host in a fixed order so the result
// does not depend on scheduling.
constexpr int kHist = 12;
__global__ void __launch_bounds__(256)
k_history(Geom g, const double* __restrict__ u, const double* __restrict__ b1,
          const double* __restrict__ b2, const double* __restrict__ b3,
          const double* __restrict__ phi, const BlockGeo* geo, int mhd, double* part) {
  const int t = blockIdx.x * blockDim.x + threadIdx.x;
  double s[kHist];
#pragma unroll
  for (int n = 0; n < kHist; ++n) s[n] = 0.0;
  if (t < g.nx1 * g.nx2) {
    const int jj = t / g.nx1, i = g.is + t - jj * g.nx1, j = g.js + jj;
    const int k = g.ks + blockIdx.y, b = blockIdx.z;
    const BlockGeo ge = geo[b];
    const double vol = ge.dx[0] * ge.dx[1] * ge.dx[2];
    const int64_t c = cidx(g, k, j, i);
    const double* ub = u + (int64_t)b * NHYD * g.ncell;
    const double d = ub[c], mx = ub[g.ncell + c], my = ub[2 * g.ncell + c],
                 mz = ub[3 * g.ncell + c], e = ub[4 * g.ncell + c];
    s[0] = vol * d;
    s[1] = vol * mx;
    s[2] = vol * my;
    s[3] = vol * mz;
    s[4] = vol * 0.5 * (mx * mx) / d;
    s[5] = vol * 0.5 * (my * my) / d;
    s[6] = vol * 0.5 * (mz * mz) / d;
    s[7] = vol * e;
    if (phi) s[8] = vol * 0.5 * d * phi[(int64_t)b * g.ncell + c];
    if (mhd) {
      const double c1 = 0.5 * b1[(int64_t)b * g.nf1 + f1idx(g, k, j, i)] +
                        0.5 * b1[(int64_t)b * g.nf1 + f1idx(g, k, j, i + 1)];
      const double c2 = 0.5 * b2[(int64_t)b * g.nf2 + f2idx(g, k, j, i)] +
                        0.5 * b2[(int64_t)b * g.nf2 + f2idx(g, k, j + 1, i)];
      const double c3 = 0.5 * b3[(int64_t)b * g.nf3 + f3idx(g, k, j, i)] +
                        0.5 * b3[(int64_t)b * g.nf3 + f3idx(g, k + 1, j, i)];
      s[9] = vol * 0.5 * c1 * c1;
      s[10] = vol * 0.5 * c2 * c2;
      s[11] = vol * 0.5 * c3 * c3;
    }
  }
  __shared__ double sh[8][kHist];
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
#pragma unroll
  for (int n = 0; n < kHist; ++n) {
    double v = s[n];
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    if (lane == 0) sh[wid][n] = v;
  }
  __syncthreads();
  if (threadIdx.x < kHist) {
    double v = 0.0;
    for (int w = 0; w < (int)(blockDim.x >> 5); ++w) v += sh[w][threadIdx.x];
    const int64_t blk = ((int64_t)blockIdx.z * gridDim.y + blockIdx.y) * gridDim.x + blockIdx.x;
    part[blk * kHist + threadIdx.x] = v;
  }
}

// Stage weights of the low-storage integrators without orbital advection
// (reference src/task_list/time_integrator.cpp:100-600).
struct Integrator {
  int nstages;
  double delta[3], g1[3], g2[3], beta[3];
};
bool make_integrator(int id, Integrator* it) {
  std::memset(it, 0, sizeof(*it));
  switch (id) {
    case ATHG_VL2:
      *it = {2, {1.0, 0.0, 0}, {0.0, 0.0, 0}, {1.0, 1.0, 0}, {0.5, 1.0, 0}};
      return true;
    case ATHG_RK1:
      *it = {1, {1.0, 0, 0}, {0.0, 0, 0}, {1.0, 0, 0}, {1.0, 0, 0}};
      return true;
    case ATHG_RK2:
      *it = {2, {1.0, 0.0, 0}, {0.0, 0.5, 0}, {1.0, 0.5, 0}, {1.0, 0.5, 0}};
      return true;
    case ATHG_RK3:
      *it = {3, {1.0, 0.0, 0.0}, {0.0, 0.25, 0.66666666666666667},
             {1.0, 0.75, 0.33333333333333333}, {1.0, 0.25, 0.66666666666666667}};
      return true;
    default:
      return false;
  }
}

}  // namespace

namespace athg {
void set_last_error(const std::string& s) { g_err = s; }
}  // namespace athg

struct athg_ctx {
  athg_config cfg{};
  Integrator integ{};
  Geom g{};
  int nb = 0;
  cudaStream_t st = nullptr;
  // pool
  double *u = nullptr, *u1 = nullptr, *b1 = nullptr, *b2 = nullptr, *b3 = nullptr;
  double *r1 = nullptr, *r2 = nullptr, *r3 = nullptr;
  void *w = nullptr, *bcc = nullptr, *flx[3] = {nullptr, nullptr, nullptr}, *edge = nullptr;
  float* cce = nullptr;  // mixed MHD: cell-centred EMF written by the primitive recovery
  float2* cce_df = nullptr;  // double-float MHD: cell-centred EMF as pairs [nb][3][cells]
  float2* wpair_df = nullptr;  // double-float: W and bcc as pairs [nb][5 or 8][cells]
  BlockGeo* geo = nullptr;
  void* coef = nullptr;        // PLM coefficients in the flux precision
  void* dxT = nullptr;         // cell widths in the flux precision
  MixedGeo* mg = nullptr;      // per-block widths of the mixed-path update
  float* dtf = nullptr;        // dt in FP32 (mixed path)
  float* bf32[3] = {nullptr, nullptr, nullptr};  // FP32 face-field copies (mixed MHD)
  int* nbr = nullptr;
  double* scal = nullptr;  // [0] time, [1] dt, [2] ncycle (as long long), [3] dtmin bits,
                           // [4..8] sums, [9] div-b bits
  std::vector<athg_block> blocks;
  std::vector<double> coords;  // host copies of x?f arrays owned by the context
  cudaGraph_t graph = nullptr;
  cudaGraphExec_t gexec = nullptr;
  // fused mixed VL2 path: the state alternates between (u, b) and (u1, r) every cycle,
  // one captured cycle per direction; FP64 ghosts are refreshed only when read
  bool fused_ok = true;        // cleared for good by the single-step entry points
  bool ghosts_stale = false;
  cudaGraph_t graph2 = nullptr;
  cudaGraphExec_t gexec2 = nullptr;
  const double* graph_src = nullptr;  // state buffer the first captured cycle reads
  FluxTune tune[4];     // launch shape of the flux sweeps, per reconstruction order 1..3
  bool tuned = false;   // autotuned (or set by the caller)
  int launches_per_cycle = 0;
  int counting = 0;
  // self-gravity (SELF_GRAVITY_ENABLED == 2): coupled multigrid solver, 4 pi G, the
  // potential of every block [nb][cells] and each block's offset in the root grid
  athg_mg* grav = nullptr;
  double four_pi_G = 0.0;
  double* phi = nullptr;
  float2* phi2 = nullptr;  // mixed path: the same potential as FP32 pairs hi + lo
  int* boff = nullptr;
  // FFT self-gravity (SELF_GRAVITY_ENABLED == 1) in place of the multigrid, and the
  // turbulence driver; both transform the whole mesh (blocks placed by boff)
  athg::FftGravity* fgrav = nullptr;
  athg::Turb* turb = nullptr;
  // multi-level mesh (static refinement): work lists, coarse buffers (FP64 path only)
  athg::SmrDevice* smr = nullptr;
  // adaptive refinement (FP64, periodic): criterion and counters; the root mesh of the
  // last athg_set_*mesh call; per-block criterion values on the device
  bool amr = false;
  athg_amr_config amrc{};
  std::vector<int> amr_deref;
  athg_mesh mesh{};
  unsigned long long* amr_bits = nullptr;
  // mixed precision on a multi-level mesh: FP64 scratch primitives and cell-centred field
  // the level-boundary lists prolongate through (the working W and bcc are FP32)
  double* smr_w64 = nullptr;
  double* smr_bcc64 = nullptr;
  // single-pass mixed VL2 MHD stage (athg_single_pass.cu): a second set of FP32 working
  // arrays (stage 1 reads the first and writes the second, stage 2 the reverse), the TMA
  // descriptors of both sets' W and bcc, and the k-segments per thread block (autotuned)
  float *w2 = nullptr, *bcc2 = nullptr, *bf32b[3] = {nullptr, nullptr, nullptr};
  athg::SinglePassMaps* spm = nullptr;  // [2]: set 1, set 2
  bool sp_ready = false;
  bool sp_on = false;     // athg_set_stage_kernel(ctx, 1, ...): one launch per stage
  bool sp_tuned = false;  // k-segments autotuned (or set by the caller)
  int sp_nseg = 1;
  // outflow physical boundaries on the non-periodic axes of a uniform mesh (FP64 arrays)
  bool outflow = false;
  // athg_cycle_timing: events recorded between launch groups, with their names
  std::vector<std::pair<std::string, cudaEvent_t>>* tev = nullptr;
  bool mixed() const { return cfg.precision == ATHG_MIXED; }
  // FP64 arrays and FP64 update, reconstruction + Riemann fluxes + corner EMFs in double-float
  bool dfloat() const { return cfg.precision == ATHG_DFLOAT; }
};

namespace {

template <typename T>
StagePtrs<T> ptrs(athg_ctx* c) {
  StagePtrs<T> p;
  p.u = c->u; p.u1 = c->u1;
  p.b1 = c->b1; p.b2 = c->b2; p.b3 = c->b3;
  p.r1 = c->r1; p.r2 = c->r2; p.r3 = c->r3;
  p.w = (T*)c->w; p.bcc = (T*)c->bcc;
  for (int d = 0; d < 3; ++d) p.flx[d] = (T*)c->flx[d];
  p.edge = (T*)c->edge;
  p.cce = std::is_same<T, float>::value ? (T*)c->cce : nullptr;
  p.geo = c->geo;
  p.coef = (const T*)c->coef;
  p.dxT = (const T*)c->dxT;
  p.mg = c->mg;
  p.dt = c->scal + 1;
  if constexpr (std::is_same<T, float>::value) {
    p.dtT = (const T*)c->dtf;
    for (int d = 0; d < 3; ++d) { p.bf[d] = (const T*)c->bf32[d]; p.bfw[d] = (T*)c->bf32[d]; }
  } else {
    p.dtT = (const T*)(c->scal + 1);
    p.bf[0] = (const T*)c->b1; p.bf[1] = (const T*)c->b2; p.bf[2] = (const T*)c->b3;
    for (int d = 0; d < 3; ++d) p.bfw[d] = nullptr;
  }
  return p;
}

// the device error word (bits kErr*), in the pool's scalar block
unsigned int* err_word(const athg_ctx* c) { return reinterpret_cast<unsigned int*>(c->scal + 12); }

// reads and clears the device error word (after the stream was synchronised)
int device_errors(athg_ctx* c) {
  unsigned int w = 0;
  CK(cudaMemcpyAsync(&w, err_word(c), sizeof(w), cudaMemcpyDeviceToHost, c->st));
  CK(cudaStreamSynchronize(c->st));
  if (!w) return ATHG_OK;
  CK(cudaMemsetAsync(err_word(c), 0, sizeof(w), c->st));
  std::string m = "device error word:";
  if (w & athg::kErrTmaTimeout) m += " a TMA load of the single-pass stage timed out;";
  if (w & athg::kErrTimeStep) m += " the new time step is not a positive finite number;";
  if (w & athg::kErrNonFinite) m += " a non-finite density or pressure was produced;";
  return fail(ATHG_ERR_DEVICE, m);
}

Phys phys(const athg_ctx* c) {
  return Phys{c->cfg.gamma, c->cfg.dfloor, c->cfg.pfloor, c->cfg.gamma - 1.0,
              split_ff(c->cfg.gamma - 1.0), split_ff(c->cfg.pfloor), (float)c->cfg.gamma,
              (float)c->cfg.dfloor, (float)c->cfg.pfloor};
}

void free_pool(athg_ctx* c) {
  void* ps[] = {c->u, c->u1, c->b1, c->b2, c->b3, c->r1, c->r2, c->r3, c->edge, c->cce, c->w,
                c->bcc, c->flx[0], c->flx[1], c->flx[2], c->geo, c->coef, c->nbr, c->scal,
                c->dxT, c->mg, c->dtf, c->bf32[0], c->bf32[1], c->bf32[2]};
  for (void* p : ps)
    if (p) cudaFree(p);
  c->u = c->u1 = c->b1 = c->b2 = c->b3 = c->r1 = c->r2 = c->r3 = nullptr;
  c->w = c->bcc = c->flx[0] = c->flx[1] = c->flx[2] = c->edge = nullptr;
  c->cce = nullptr;
  c->geo = nullptr; c->coef = nullptr; c->nbr = nullptr; c->scal = nullptr;
  c->dxT = nullptr; c->mg = nullptr; c->dtf = nullptr;
  c->bf32[0] = c->bf32[1] = c->bf32[2] = nullptr;
  if (c->gexec) cudaGraphExecDestroy(c->gexec);
  if (c->graph) cudaGraphDestroy(c->graph);
  if (c->gexec2) cudaGraphExecDestroy(c->gexec2);
  if (c->graph2) cudaGraphDestroy(c->graph2);
  c->gexec = nullptr; c->graph = nullptr;
  c->gexec2 = nullptr; c->graph2 = nullptr;
  c->ghosts_stale = false;
  if (c->phi) cudaFree(c->phi);
  if (c->phi2) cudaFree(c->phi2);
  if (c->boff) cudaFree(c->boff);
  c->phi = nullptr; c->phi2 = nullptr; c->boff = nullptr;
  if (c->grav) athg::mg_bind_stream(c->grav, nullptr);
  c->grav = nullptr;
  athg::fftgrav_destroy(c->fgrav);
  c->fgrav = nullptr;
  athg::turb_destroy(c->turb);
  c->turb = nullptr;
  athg::smr_destroy(c->smr);
  c->smr = nullptr;
  if (c->amr_bits) cudaFree(c->amr_bits);
  c->amr_bits = nullptr;
  if (c->smr_w64) cudaFree(c->smr_w64);
  if (c->smr_bcc64) cudaFree(c->smr_bcc64);
  c->smr_w64 = c->smr_bcc64 = nullptr;
  void* sp[] = {c->w2, c->bcc2, c->bf32b[0], c->bf32b[1], c->bf32b[2], c->cce_df,
                c->wpair_df};
  c->cce_df = nullptr;
  c->wpair_df = nullptr;
  for (void* q : sp)
    if (q) cudaFree(q);
  c->w2 = c->bcc2 = nullptr;
  c->bf32b[0] = c->bf32b[1] = c->bf32b[2] = nullptr;
  delete[] c->spm;
  c->spm = nullptr;
  c->sp_ready = false;
  c->nb = 0;
}

// the block pool as the SMR work lists see it
SmrPool smr_pool_of(athg_ctx* c) {
  SmrPool P = athg::smr_pool(c->smr);
  P.u = c->u;
  P.b1 = c->b1; P.b2 = c->b2; P.b3 = c->b3;
  P.nflx = c->cfg.magnetic ? 8 : 5;
  if (c->mixed()) {
    P.w = c->smr_w64;
    P.bcc = c->smr_bcc64;
    for (int d = 0; d < 3; ++d) P.flx32[d] = (float*)c->flx[d];
    P.edge32 = (float*)c->edge;
  } else {
    P.w = (double*)c->w;
    P.bcc = (double*)c->bcc;
    for (int d = 0; d < 3; ++d) P.flx[d] = (double*)c->flx[d];
    P.edge = (double*)c->edge;
  }
  P.gamma = c->cfg.gamma; P.dfloor = c->cfg.dfloor; P.pfloor = c->cfg.pfloor;
  return P;
}

int launch_ghosts(athg_ctx* c) {
  if (c->smr) {  // ghost fill across refinement levels and prolongation
    c->counting += athg::smr_fill(c->smr, smr_pool_of(c), c->st);
    CKL();
    return ATHG_OK;
  }
  GhostPtrs gp{c->u, c->b1, c->b2, c->b3, c->nbr, NHYD, c->cfg.magnetic};
  const Geom& g = c->g;
  dim3 grid((unsigned)((ghost_shell_size(g) + 255) / 256), (unsigned)c->nb);
  k_ghost_same_level<<<grid, 256, 0, c->st>>>(g, gp);
  c->counting += 1;
  CKL();
  return ATHG_OK;
}

bool df_fast(const athg_ctx* c);

int launch_fluxes(athg_ctx* c, int order) {
  bool mhd = c->cfg.magnetic != 0;
  if (c->mixed())
    Launcher<float>::fluxes(c->g, ptrs<float>(c), mhd, c->cfg.rsolver, order, phys(c),
                            c->tune[order], c->st);
  else if (c->dfloat())
    athg::df_fluxes(c->g, ptrs<double>(c), mhd, c->cfg.rsolver, order, phys(c), c->wpair_df,
                    df_fast(c), c->st);
  else
    Launcher<double>::fluxes(c->g, ptrs<double>(c), mhd, c->cfg.rsolver, order, phys(c),
                             c->tune[order], c->st);
  c->counting += 3;
  // SendFluxCorrection / ReceiveFluxCorrection (time_integrator.cpp: SEND_HYDFLX, RECV_HYDFLX)
  if (c->smr) c->counting += athg::smr_correct_flux(c->smr, smr_pool_of(c), c->st);
  CKL();
  return ATHG_OK;
}

int launch_corner(athg_ctx* c) {
  if (!c->cfg.magnetic) return ATHG_OK;
  if (c->mixed()) Launcher<float>::corner_emf(c->g, ptrs<float>(c), c->st);
  else if (c->dfloat())
    athg::df_corner_emf(c->g, ptrs<double>(c), c->cce_df, c->wpair_df, df_fast(c), c->st);
  else Launcher<double>::corner_emf(c->g, ptrs<double>(c), c->st);
  c->counting += 1;
  // EMF correction at block boundaries (time_integrator.cpp: SEND_FLDFLX, RECV_FLDFLX)
  if (c->smr) c->counting += athg::smr_correct_emf(c->smr, smr_pool_of(c), c->st);
  CKL();
  return ATHG_OK;
}

StageW stage_weights(const athg_ctx* c, int l) {
  const Integrator& it = c->integ;
  StageW sw;
  sw.delta = it.delta[l];
  sw.g1 = it.g1[l];
  sw.g2 = it.g2[l];
  sw.beta = it.beta[l];
  sw.swap = (it.g1[l] == 0.0 && it.g2[l] == 1.0) ? 1 : 0;
  sw.zero_reg = (l == 0) ? 1 : 0;
  sw.copy_reg = (sw.zero_reg && sw.delta == 1.0) ? 1 : 0;
  sw.has_delta = (sw.delta != 0.0) ? 1 : 0;
  sw.betaf = (float)sw.beta;
  return sw;
}

int launch_update(athg_ctx* c, int l) {
  StageW sw = stage_weights(c, l);
  bool mhd = c->cfg.magnetic != 0;
  if (c->mixed()) Launcher<float>::update(c->g, ptrs<float>(c), mhd, sw, c->st);
  else if (df_fast(c)) athg::df_update(c->g, ptrs<double>(c), mhd, sw, c->st);
  else Launcher<double>::update(c->g, ptrs<double>(c), mhd, sw, c->st);
  c->counting += 1;
  CKL();
  return ATHG_OK;
}

int launch_c2p(athg_ctx* c) {
  bool mhd = c->cfg.magnetic != 0;
  if (c->mixed()) Launcher<float>::c2p(c->g, ptrs<float>(c), mhd, phys(c), c->st);
  else if (df_fast(c)) athg::df_c2p(c->g, ptrs<double>(c), mhd, phys(c), c->wpair_df, c->st);
  else Launcher<double>::c2p(c->g, ptrs<double>(c), mhd, phys(c), c->st);
  c->counting += 1;
  if (c->outflow) {  // ApplyPhysicalBoundaries after the primitives (FP64 arrays)
    OutflowPtrs op{c->u, (double*)c->w, c->b1, c->b2, c->b3, (double*)c->bcc, c->nbr,
                   mhd ? 1 : 0, 1.0 / (c->cfg.gamma - 1.0)};
    const dim3 grid((unsigned)((ghost_shell_size(c->g) + 255) / 256), (unsigned)c->nb);
    k_outflow_copy<<<grid, 256, 0, c->st>>>(c->g, op);
    k_outflow_cons<<<grid, 256, 0, c->st>>>(c->g, op);
    c->counting += 2;
  }
  CKL();
  return ATHG_OK;
}

int launch_block_dt(athg_ctx* c) {
  bool mhd = c->cfg.magnetic != 0;
  unsigned long long* dm = (unsigned long long*)(c->scal + 3);
  if (c->mixed()) Launcher<float>::block_dt(c->g, ptrs<float>(c), mhd, phys(c), dm, c->st);
  else if (df_fast(c))
    athg::df_block_dt(c->g, ptrs<double>(c), mhd, phys(c), c->wpair_df, dm, c->st);
  else Launcher<double>::block_dt(c->g, ptrs<double>(c), mhd, phys(c), dm, c->st);
  c->counting += 1;
  CKL();
  return ATHG_OK;
}

int launch_end(athg_ctx* c, int advance) {
  k_end_cycle<<<1, 32, 0, c->st>>>(c->scal, c->scal + 1, (long long*)(c->scal + 2),
                                   (unsigned long long*)(c->scal + 3), c->cfg.cfl_number,
                                   c->cfg.tlim, advance, c->dtf, err_word(c));
  c->counting += 1;
  CKL();
  return ATHG_OK;
}

// Multigrid::LoadSource (multigrid/multigrid.cpp:194-233): u(IDN) of every block, times
// 4 pi G, into the interior of the solver's finest level
__global__ void k_gather_rho(Geom g, const double* __restrict__ u, const int* __restrict__ boff,
                             double* __restrict__ src, int n, double fac) {
  const int b = blockIdx.z, k = blockIdx.y;
  const int t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= g.nx1 * g.nx2) return;
  const int j = t / g.nx1, i = t - j * g.nx1;
  const double d = u[(int64_t)b * NHYD * g.ncell + cidx(g, k + g.ks, j + g.js, i + g.is)];
  const int64_t nt = n + 2;
  const int I = boff[3 * b] + i + 1, J = boff[3 * b + 1] + j + 1, K = boff[3 * b + 2] + k + 1;
  src[((int64_t)K * nt + J) * nt + I] = (fac == 1.0) ? d : d * fac;
}

// Multigrid::RetrieveResult (multigrid.cpp:269-286) with one ghost layer: the solver's
// finest level, whose ghost layer holds the final boundary fill, into every block's phi
// (and, for the mixed path's source term, into phi2 as FP32 pairs)
__global__ void k_scatter_phi(Geom g, double* __restrict__ phi, float2* __restrict__ phi2,
                              const int* __restrict__ boff, const double* __restrict__ um,
                              int n) {
  const int b = blockIdx.z, k = blockIdx.y;  // k over nx3 + 2
  const int t = blockIdx.x * blockDim.x + threadIdx.x;
  const int w1 = g.nx1 + 2, w2 = g.nx2 + 2;
  if (t >= w1 * w2) return;
  const int j = t / w1, i = t - j * w1;
  const int64_t nt = n + 2;
  const int I = boff[3 * b] + i, J = boff[3 * b + 1] + j, K = boff[3 * b + 2] + k;
  const int64_t q = (int64_t)b * g.ncell + cidx(g, k + g.ks - 1, j + g.js - 1, i + g.is - 1);
  const double v = um[((int64_t)K * nt + J) * nt + I];
  phi[q] = v;
  if (phi2) {
    const athg::ff f = athg::split_ff(v);
    phi2[q] = make_float2(f.hi, f.lo);
  }
}

bool has_gravity(const athg_ctx* c) { return c->grav || c->fgrav; }

// The double-float path without FP64 arithmetic in the update, primitive recovery and time
// step (df_update, df_c2p, df_block_dt): uniform periodic meshes without source terms, where
// nothing but those kernels writes the primitives the flux sweeps read as pairs
bool df_fast(const athg_ctx* c) {
  return c->dfloat() && !c->smr && !has_gravity(c) && !c->outflow && !c->turb;
}

// whether a cycle can be captured as a CUDA graph: no host synchronisation inside (a
// multigrid iterating to a threshold or with multipole boundaries); the FFT solve's cuFFT
// executions and kernels are captured with the rest
bool captured(const athg_ctx* c) { return !(c->grav && !athg::mg_solve_capturable(c->grav)); }

// TurbulenceDriver::Driving at the context's current time and dt
int turb_drive(athg_ctx* c) {
  double hs[2];
  CK(cudaMemcpyAsync(hs, c->scal, sizeof(hs), cudaMemcpyDeviceToHost, c->st));
  CK(cudaStreamSynchronize(c->st));
  std::string err;
  if (athg::turb_drive(c->turb, c->g, c->nb, c->u, c->boff, hs[0], hs[1], c->st, &err))
    return fail(ATHG_ERR_CUDA, err);
  c->counting += 6;
  return ATHG_OK;
}

// Offsets of every block in a mesh-wide array of n1 x n2 x n3 cells (one uniform level
// tiling it) into c->boff; the phi array of the gravity coupling is allocated with it.
int tile_blocks(athg_ctx* c, int n1, int n2, int n3) {
  const Geom& g = c->g;
  if (c->smr) return fail(ATHG_ERR_ARG, "a mesh-wide solver on a multi-level mesh is not supported");
  if (n1 % g.nx1 || n2 % g.nx2 || n3 % g.nx3)
    return fail(ATHG_ERR_ARG, "mesh size is not a multiple of the block size");
  const int64_t nbx = n1 / g.nx1, nby = n2 / g.nx2, nbz = n3 / g.nx3;
  if (nbx * nby * nbz != c->nb) return fail(ATHG_ERR_ARG, "blocks do not tile the mesh");
  std::vector<int> hb(3 * c->nb);
  std::vector<char> seen((size_t)nbx * nby * nbz, 0);
  for (int b = 0; b < c->nb; ++b) {
    const athg_block& B = c->blocks[b];
    if (B.level != c->blocks[0].level)
      return fail(ATHG_ERR_ARG, "a mesh-wide solver needs blocks of one refinement level");
    if (B.lx1 < 0 || B.lx1 >= nbx || B.lx2 < 0 || B.lx2 >= nby || B.lx3 < 0 || B.lx3 >= nbz)
      return fail(ATHG_ERR_ARG, "block location outside the mesh");
    char& f = seen[((size_t)B.lx3 * nby + B.lx2) * nbx + B.lx1];
    if (f) return fail(ATHG_ERR_ARG, "two blocks at one location");
    f = 1;
    hb[3 * b] = (int)(B.lx1 * g.nx1);
    hb[3 * b + 1] = (int)(B.lx2 * g.nx2);
    hb[3 * b + 2] = (int)(B.lx3 * g.nx3);
  }
  if (!c->boff) CK(cudaMalloc(&c->boff, sizeof(int) * 3 * c->nb));
  if (!c->phi) {
    CK(cudaMalloc(&c->phi, sizeof(double) * g.ncell * c->nb));
    CK(cudaMemsetAsync(c->phi, 0, sizeof(double) * g.ncell * c->nb, c->st));
  }
  if (c->mixed() && !c->phi2) {
    CK(cudaMalloc(&c->phi2, sizeof(float2) * g.ncell * c->nb));
    CK(cudaMemsetAsync(c->phi2, 0, sizeof(float2) * g.ncell * c->nb, c->st));
  }
  CK(cudaMemcpyAsync(c->boff, hb.data(), sizeof(int) * hb.size(), cudaMemcpyHostToDevice, c->st));
  CK(cudaStreamSynchronize(c->st));
  return ATHG_OK;
}

// MGGravityDriver::Solve (gravity/mg_gravity.cpp:166-211) on the context's stream, from
// the density of `ucons` (the current state, or the fused stage's output buffer)
int gravity_solve(athg_ctx* c, const double* ucons) {
  if (c->fgrav) {  // FFTGravityDriver::Solve (gravity/fft_gravity.cpp:58-100)
    std::string err;
    if (athg::fftgrav_solve(c->fgrav, c->g, c->nb, ucons, c->boff, c->phi, c->phi2, c->st,
                            &err))
      return fail(ATHG_ERR_CUDA, err);
    c->counting += 4;
    return ATHG_OK;
  }
  double *um, *src;
  int n;
  int rc = athg::mg_finest(c->grav, &um, &src, &n);
  if (rc) return rc;
  const Geom& g = c->g;
  dim3 gg((unsigned)((g.nx1 * g.nx2 + 255) / 256), (unsigned)g.nx3, (unsigned)c->nb);
  k_gather_rho<<<gg, 256, 0, c->st>>>(g, ucons, c->boff, src, n, c->four_pi_G);
  CKL();
  if ((rc = athg::mg_solve(c->grav, false, nullptr, nullptr))) return rc;
  dim3 gs((unsigned)(((g.nx1 + 2) * (g.nx2 + 2) + 255) / 256), (unsigned)(g.nx3 + 2),
          (unsigned)c->nb);
  k_scatter_phi<<<gs, 256, 0, c->st>>>(g, c->phi, c->phi2, c->boff, um, n);
  CKL();
  c->counting += 2;
  return ATHG_OK;
}

int launch_self_gravity(athg_ctx* c, int l) {
  StageW sw = stage_weights(c, l);
  bool mhd = c->cfg.magnetic != 0;
  if (c->mixed()) Launcher<float>::self_gravity(c->g, ptrs<float>(c), mhd, sw, c->phi, c->st);
  else Launcher<double>::self_gravity(c->g, ptrs<double>(c), mhd, sw, c->phi, c->st);
  c->counting += 1;
  CKL();
  return ATHG_OK;
}

bool fused(const athg_ctx* c) {
  return c->fused_ok && c->mixed() && c->cfg.integrator == ATHG_VL2 && !c->smr;
}

// The single-pass stage kernel (opt-in: athg_set_stage_kernel) covers the fused path for
// MHD with PLM (donor cell in the first VL2 stage), HLLD or HLLE, on meshes whose blocks it
// tiles
bool single_pass(const athg_ctx* c) {
  return fused(c) && !has_gravity(c) && c->cfg.magnetic && c->cfg.xorder == 2 &&
         (c->cfg.rsolver == ATHG_HLLD || c->cfg.rsolver == ATHG_HLLE) && c->sp_on &&
         athg::single_pass_fits(c->g, 1);
}

// the second set of FP32 working arrays and the TMA descriptors of both sets (allocates:
// called outside stream capture)
int sp_prepare(athg_ctx* c) {
  if (c->sp_ready) return ATHG_OK;
  const Geom& g = c->g;
  if (int e = athg::single_pass_setup())
    return fail(ATHG_ERR_CUDA, std::string("single-pass kernel attributes: ") +
                                   cudaGetErrorString((cudaError_t)e));
  const size_t nb = (size_t)c->nb;
  CK(cudaMalloc(&c->w2, sizeof(float) * NHYD * g.ncell * nb));
  CK(cudaMalloc(&c->bcc2, sizeof(float) * 3 * g.ncell * nb));
  const int64_t nf[3] = {g.nf1, g.nf2, g.nf3};
  for (int d = 0; d < 3; ++d) CK(cudaMalloc(&c->bf32b[d], sizeof(float) * nf[d] * nb));
  // the second set starts as a copy (its ghost zones are rewritten after every stage)
  CK(cudaMemcpyAsync(c->w2, c->w, sizeof(float) * NHYD * g.ncell * nb, cudaMemcpyDeviceToDevice, c->st));
  CK(cudaMemcpyAsync(c->bcc2, c->bcc, sizeof(float) * 3 * g.ncell * nb, cudaMemcpyDeviceToDevice, c->st));
  for (int d = 0; d < 3; ++d)
    CK(cudaMemcpyAsync(c->bf32b[d], c->bf32[d], sizeof(float) * nf[d] * nb,
                       cudaMemcpyDeviceToDevice, c->st));
  c->spm = new athg::SinglePassMaps[2];
  std::string err;
  if (athg::single_pass_maps((const float*)c->w, (const float*)c->bcc, g, &c->spm[0], &err) ||
      athg::single_pass_maps(c->w2, c->bcc2, g, &c->spm[1], &err))
    return fail(ATHG_ERR_CUDA, err);
  c->sp_ready = true;
  return ATHG_OK;
}

// one stage of the single-pass kernel: stage 1 reads FP32 set 1 and writes set 2, stage 2
// the reverse, so after a whole VL2 cycle the current W is in set 1 again; then the ghost
// exchange of the set just written. order_override > 0 replaces the stage's reconstruction
// order (the autotuner times the second stage's PLM kernel in the first stage's direction,
// which writes only scratch: the other state buffer and FP32 set 2).
int launch_single_pass(athg_ctx* c, int l, bool dt_too, int order_override = 0) {
  const bool first = (l == 0);
  const int order = order_override > 0 ? order_override : (first ? 1 : c->cfg.xorder);
  StagePtrs<float> p = ptrs<float>(c);
  float* set1w = (float*)c->w;
  float* set1b = (float*)c->bcc;
  float* const set1f[3] = {c->bf32[0], c->bf32[1], c->bf32[2]};
  float* const set2f[3] = {c->bf32b[0], c->bf32b[1], c->bf32b[2]};
  if (!first) {
    p.w = c->w2; p.bcc = c->bcc2;
    for (int d = 0; d < 3; ++d) p.bf[d] = c->bf32b[d];
  }
  StateBufs sb;
  sb.u_in = c->u; sb.u_out = c->u1;
  sb.b_in[0] = c->b1; sb.b_in[1] = c->b2; sb.b_in[2] = c->b3;
  sb.b_out[0] = c->r1; sb.b_out[1] = c->r2; sb.b_out[2] = c->r3;
  const int e = athg::single_pass_launch(
      c->spm[first ? 0 : 1], c->g, p, first ? c->w2 : set1w, first ? c->bcc2 : set1b,
      first ? set2f : set1f, sb, stage_weights(c, l), phys(c),
      dt_too ? (unsigned long long*)(c->scal + 3) : nullptr, err_word(c), order,
      c->cfg.rsolver == ATHG_HLLD ? HLLD : HLLE, c->sp_nseg, c->st);
  if (e) return fail(ATHG_ERR_CUDA, std::string("single-pass stage: ") +
                                        cudaGetErrorString((cudaError_t)e));
  c->counting += 1;
  return ATHG_OK;
}

int launch_ghosts_set(athg_ctx* c, float* w, float* bcc, float* const bf[3], float* cce) {
  const Geom& g = c->g;
  GhostPtrs32 gp;
  const bool mhd = c->cfg.magnetic != 0;
  gp.cell[0] = w; gp.ncomp[0] = NHYD;
  gp.cell[1] = mhd ? bcc : nullptr; gp.ncomp[1] = 3;
  gp.cell[2] = mhd ? cce : nullptr; gp.ncomp[2] = 3;
  for (int d = 0; d < 3; ++d) gp.face[d] = mhd ? bf[d] : nullptr;
  gp.nbr = c->nbr;
  dim3 grid((unsigned)((ghost_shell_size(g) + 255) / 256), (unsigned)c->nb);
  if (mhd) k_ghost_f32<true><<<grid, 256, 0, c->st>>>(g, gp);
  else k_ghost_f32<false><<<grid, 256, 0, c->st>>>(g, gp);
  c->counting += 1;
  CKL();
  return ATHG_OK;
}

// swap the two state buffers (after a fused cycle the new state is in (u1, r))
void swap_state(athg_ctx* c) {
  std::swap(c->u, c->u1);
  std::swap(c->b1, c->r1);
  std::swap(c->b2, c->r2);
  std::swap(c->b3, c->r3);
}

// dt_too: the last stage also reduces the CFL time step (k_block_dt folded in)
int launch_update_c2p(athg_ctx* c, int l, bool dt_too) {
  StageW sw = stage_weights(c, l);
  StateBufs sb;
  sb.u_in = c->u; sb.u_out = c->u1;
  sb.b_in[0] = c->b1; sb.b_in[1] = c->b2; sb.b_in[2] = c->b3;
  sb.b_out[0] = c->r1; sb.b_out[1] = c->r2; sb.b_out[2] = c->r3;
  Launcher<float>::update_c2p(c->g, ptrs<float>(c), c->cfg.magnetic != 0, sw, phys(c), sb,
                              dt_too ? (unsigned long long*)(c->scal + 3) : nullptr,
                              has_gravity(c) ? c->phi2 : nullptr, c->st);
  c->counting += 1;
  CKL();
  return ATHG_OK;
}

int launch_ghosts_f32(athg_ctx* c) {
  float* const bf[3] = {c->bf32[0], c->bf32[1], c->bf32[2]};
  return launch_ghosts_set(c, (float*)c->w, (float*)c->bcc, bf, c->cce);
}

// FP64 ghost zones of the current state, when a fused cycle left them behind
int refresh_ghosts(athg_ctx* c) {
  if (!c->ghosts_stale) return ATHG_OK;
  int rc = launch_ghosts(c);
  if (rc) return rc;
  c->ghosts_stale = false;
  return ATHG_OK;
}

void drop_graphs(athg_ctx* c) {
  if (c->gexec) cudaGraphExecDestroy(c->gexec);
  if (c->graph) cudaGraphDestroy(c->graph);
  if (c->gexec2) cudaGraphExecDestroy(c->gexec2);
  if (c->graph2) cudaGraphDestroy(c->graph2);
  c->gexec = nullptr; c->graph = nullptr; c->gexec2 = nullptr; c->graph2 = nullptr;
  c->graph_src = nullptr;
}

// the single-step entry points work on the unfused path from here on
int leave_fused(athg_ctx* c) {
  int rc = refresh_ghosts(c);
  if (rc) return rc;
  if (c->fused_ok) {
    c->fused_ok = false;
    drop_graphs(c);
  }
  return ATHG_OK;
}

// an event after the launch group `what` of stage `stage` (athg_cycle_timing only)
void mark(athg_ctx* c, int stage, const char* what) {
  if (!c->tev) return;
  cudaEvent_t e;
  if (cudaEventCreate(&e) != cudaSuccess) return;
  cudaEventRecord(e, c->st);
  c->tev->push_back(std::make_pair("stage " + std::to_string(stage) + ": " + what, e));
}

int do_stage(athg_ctx* c, int stage) {
  const int l = stage - 1;
  int order = (c->cfg.integrator == ATHG_VL2 && l == 0) ? 1 : c->cfg.xorder;
  int rc;
  if (single_pass(c) && c->sp_ready) {
    if ((rc = launch_single_pass(c, l, stage == c->integ.nstages))) return rc;
    mark(c, stage, "single-pass stage (k_single_pass)");
    if (l == 0) {
      float* const bf[3] = {c->bf32b[0], c->bf32b[1], c->bf32b[2]};
      rc = launch_ghosts_set(c, c->w2, c->bcc2, bf, nullptr);
    } else {
      float* const bf[3] = {c->bf32[0], c->bf32[1], c->bf32[2]};
      rc = launch_ghosts_set(c, (float*)c->w, (float*)c->bcc, bf, nullptr);
    }
    if (rc) return rc;
    mark(c, stage, "ghost exchange");
    c->ghosts_stale = true;
    return ATHG_OK;
  }
  if (fused(c)) {
    if ((rc = launch_fluxes(c, order))) return rc;
    mark(c, stage, "flux sweeps");
    if ((rc = launch_corner(c))) return rc;
    mark(c, stage, "corner EMF");
    if ((rc = launch_update_c2p(c, l, stage == c->integ.nstages))) return rc;
    mark(c, stage, "update + primitives (k_update_c2p)");
    if ((rc = launch_ghosts_f32(c))) return rc;
    mark(c, stage, "ghost exchange");
    c->ghosts_stale = true;
    // the potential of the new state for the next stage (main.cpp:461-466)
    if (has_gravity(c) && (rc = gravity_solve(c, c->u1))) return rc;
    if (has_gravity(c)) mark(c, stage, "gravity solve");
    return ATHG_OK;
  }
  if ((rc = launch_fluxes(c, order))) return rc;
  mark(c, stage, "flux sweeps");
  if ((rc = launch_corner(c))) return rc;
  mark(c, stage, "corner EMF");
  if ((rc = launch_update(c, l))) return rc;
  mark(c, stage, "update (k_update)");
  // AddSourceTerms (time_integrator.cpp:1655-1676); every stage here is a main stage
  if (has_gravity(c) && (rc = launch_self_gravity(c, l))) return rc;
  if (has_gravity(c)) mark(c, stage, "self-gravity source");
  if ((rc = launch_ghosts(c))) return rc;
  mark(c, stage, "ghost exchange");
  if ((rc = launch_c2p(c))) return rc;
  mark(c, stage, "primitives (k_c2p)");
  if (has_gravity(c) && (rc = gravity_solve(c, c->u))) return rc;  // main.cpp:461-466
  if (has_gravity(c)) mark(c, stage, "gravity solve");
  if (stage == c->integ.nstages) {
    if ((rc = launch_block_dt(c))) return rc;
    mark(c, stage, "time step");
  }
  return ATHG_OK;
}

int do_cycle(athg_ctx* c) {
  for (int s = 1; s <= c->integ.nstages; ++s) {
    int rc = do_stage(c, s);
    if (rc) return rc;
  }
  int rc = launch_end(c, 1);
  mark(c, c->integ.nstages, "end of cycle");
  return rc;
}

int need_pool(const athg_ctx* c) {
  if (!c) return fail(ATHG_ERR_ARG, "null context");
  if (c->nb <= 0) return fail(ATHG_ERR_STATE, "no blocks: call athg_set_blocks first");
  return ATHG_OK;
}

// Captures one whole cycle on the context stream into a CUDA graph (once); the
// graph reads dt/time from device memory, so the same graph serves every cycle.
int capture_cycle(athg_ctx* c, cudaGraph_t* graph, cudaGraphExec_t* exec) {
  CK(cudaStreamBeginCapture(c->st, cudaStreamCaptureModeThreadLocal));
  c->counting = 0;
  const bool stale = c->ghosts_stale;
  int rc = do_cycle(c);
  c->ghosts_stale = stale;  // capturing runs nothing
  cudaGraph_t gr = nullptr;
  cudaError_t e = cudaStreamEndCapture(c->st, &gr);
  if (rc) {
    if (gr) cudaGraphDestroy(gr);
    return rc;
  }
  if (e != cudaSuccess)
    return fail(ATHG_ERR_CUDA, std::string("graph capture: ") + cudaGetErrorString(e));
  *graph = gr;
  c->launches_per_cycle = c->counting;
  CK(cudaGraphInstantiate(exec, gr, 0));
  return ATHG_OK;
}

// Autotuner of the flux sweeps' launch shape (threads per block of the x1 and marching
// sweeps, faces per marching segment), one shape per reconstruction order the integrator
// uses: every candidate runs the three sweeps of one stage on the context's own state
// (they only write the flux arrays) three times, timed with CUDA events on the context's
// stream; the fastest median wins. Mixed path only (the FP64
// path is the reference-order check, not the fast path); runs once, before the first
// captured cycle.
int autotune_single_pass(athg_ctx* c);

int autotune(athg_ctx* c) {
  if (!c->mixed()) return ATHG_OK;
  cudaStreamCaptureStatus cs = cudaStreamCaptureStatusNone;
  CK(cudaStreamIsCapturing(c->st, &cs));
  if (cs != cudaStreamCaptureStatusNone) return ATHG_OK;
  if (single_pass(c)) {
    int rc = sp_prepare(c);
    if (rc) return rc;
    if (c->sp_tuned) return ATHG_OK;
    c->sp_tuned = true;
    return autotune_single_pass(c);
  }
  if (c->tuned) return ATHG_OK;
  c->tuned = true;
  const int tpbs[2] = {64, 128}, segs[5] = {4, 8, 16, 32, 0};
  cudaEvent_t e0, e1;
  CK(cudaEventCreate(&e0));
  CK(cudaEventCreate(&e1));
  const bool mhd = c->cfg.magnetic != 0;
  const int saved = c->counting;
  int rc = ATHG_OK;
  // each reconstruction order the integrator uses (VL2: donor cell, then xorder) has its
  // own registers per thread, so its own best shape
  const int orders[2] = {c->cfg.integrator == ATHG_VL2 ? 1 : c->cfg.xorder, c->cfg.xorder};
  for (int oi = 0; oi < 2 && !rc; ++oi) {
    const int order = orders[oi];
    if (oi == 1 && order == orders[0]) break;
    FluxTune best = c->tune[order];
    float best_ms = 1e30f;
    for (int a = 0; a < 2 && !rc; ++a)
      for (int m = 0; m < 2 && !rc; ++m)
        for (int q = 0; q < 5 && !rc; ++q) {
          FluxTune t;
          t.x1_tpb = tpbs[a]; t.march_tpb = tpbs[m]; t.seg = segs[q];
          float ms[3];
          for (int r = 0; r < 3; ++r) {
            cudaEventRecord(e0, c->st);
            Launcher<float>::fluxes(c->g, ptrs<float>(c), mhd, c->cfg.rsolver, order, phys(c),
                                    t, c->st);
            cudaEventRecord(e1, c->st);
            if (cudaEventSynchronize(e1) != cudaSuccess || cudaGetLastError() != cudaSuccess) {
              rc = fail(ATHG_ERR_CUDA, "autotune launch failed");
              break;
            }
            cudaEventElapsedTime(&ms[r], e0, e1);
          }
          if (rc) break;
          std::sort(ms, ms + 3);
          if (ms[1] < best_ms) { best_ms = ms[1]; best = t; }
        }
    if (!rc) c->tune[order] = best;
  }
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  c->counting = saved;
  return rc;
}

// k-segments per thread block of the single-pass stage: each candidate (1, 2, 4 segments
// where they divide the block) runs the PLM kernel on the context's own state three times
// in the first stage's direction (reading FP32 set 1, writing only the other state buffer
// and FP32 set 2, which the next real stage overwrites), timed with CUDA events; the
// fastest median wins.
int autotune_single_pass(athg_ctx* c) {
  cudaEvent_t e0, e1;
  CK(cudaEventCreate(&e0));
  CK(cudaEventCreate(&e1));
  const int saved = c->counting;
  int best = 1;
  float best_ms = 1e30f;
  int rc = ATHG_OK;
  for (int nseg = 1; nseg <= 4 && !rc; nseg *= 2) {
    if (!athg::single_pass_fits(c->g, nseg)) continue;
    c->sp_nseg = nseg;
    float ms[3];
    for (int r = 0; r < 3 && !rc; ++r) {
      cudaEventRecord(e0, c->st);
      rc = launch_single_pass(c, 0, false, c->cfg.xorder);
      cudaEventRecord(e1, c->st);
      if (!rc && (cudaEventSynchronize(e1) != cudaSuccess || cudaGetLastError() != cudaSuccess))
        rc = fail(ATHG_ERR_CUDA, "autotune launch failed");
      if (!rc) cudaEventElapsedTime(&ms[r], e0, e1);
    }
    if (rc) break;
    std::sort(ms, ms + 3);
    if (ms[1] < best_ms) { best_ms = ms[1]; best = nseg; }
  }
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  c->counting = saved;
  c->sp_nseg = best;
  return rc;
}

int build_graph(athg_ctx* c) {
  if (c->gexec) return ATHG_OK;
  int trc = autotune(c);
  if (trc) return trc;
  int rc = capture_cycle(c, &c->graph, &c->gexec);
  if (rc) return rc;
  c->graph_src = c->u;
  if (fused(c)) {  // the cycle that starts from the other buffer
    swap_state(c);
    rc = capture_cycle(c, &c->graph2, &c->gexec2);
    swap_state(c);
    if (rc) return rc;
  }
  return ATHG_OK;
}

// one whole cycle from the captured graphs; in the fused path the new state is then in
// the other buffer
int run_cycle_graph(athg_ctx* c) {
  if (fused(c)) {
    CK(cudaGraphLaunch(c->u == c->graph_src ? c->gexec : c->gexec2, c->st));
    swap_state(c);
    c->ghosts_stale = true;
  } else {
    CK(cudaGraphLaunch(c->gexec, c->st));
  }
  return ATHG_OK;
}

// one whole cycle launched kernel by kernel (a cycle that cannot be captured: a multigrid
// iterating to a threshold or with multipole boundaries); in the fused path the new state
// is then in the other buffer, as after run_cycle_graph
int run_cycle_direct(athg_ctx* c) {
  int rc = autotune(c);
  if (rc) return rc;
  if ((rc = do_cycle(c))) return rc;
  if (fused(c)) {
    swap_state(c);
    c->ghosts_stale = true;
  }
  return ATHG_OK;
}

// mesh/mesh.hpp:389-405 and :467-488: symmetric logical position, uniform generator
double gen_rx(int64_t index, int64_t nrange) {
  int64_t noffset = index - nrange / 2;
  int64_t noffset_ceil = index - (nrange + 1) / 2;
  return static_cast<double>(noffset + noffset_ceil) / (2.0 * nrange);
}
double gen_x(double rx, double xmin, double xmax) {
  return 0.5 * (xmin + xmax) + (rx * xmax - rx * xmin);
}

// ---- multi-level meshes ----------------------------------------------------------------
using LocKey = std::tuple<int, int64_t, int64_t, int64_t>;

// Leaves of a root grid refined by <refinementN> regions (Mesh::Mesh, mesh/mesh.cpp:334-462:
// logical range of each region at its level widened to whole parents, AddMeshBlock), then
// refined further until neighbouring leaves differ by at most one level (the balance
// MeshBlockTree::Refine keeps, mesh/meshblock_tree.cpp)
int refined_leaves(const int nmx[3], const int nrb[3], const double lo[3], const double hi[3],
                   int nreg, const athg_region* reg, std::vector<SmrLoc>* out) {
  std::set<LocKey> leaves;
  for (int k = 0; k < nrb[2]; ++k)
    for (int j = 0; j < nrb[1]; ++j)
      for (int i = 0; i < nrb[0]; ++i) leaves.insert(LocKey(0, i, j, k));
  auto refine = [&](const LocKey& key) {
    leaves.erase(key);
    const int l = std::get<0>(key);
    for (int c8 = 0; c8 < 8; ++c8)
      leaves.insert(LocKey(l + 1, 2 * std::get<1>(key) + (c8 & 1),
                           2 * std::get<2>(key) + ((c8 >> 1) & 1), 2 * std::get<3>(key) + (c8 >> 2)));
  };
  auto add_block = [&](int L, const int64_t x[3]) {
    for (int lv = 0; lv < L; ++lv) {
      const int sh = L - lv;
      LocKey a(lv, x[0] >> sh, x[1] >> sh, x[2] >> sh);
      if (leaves.count(a)) refine(a);
    }
  };
  for (int r = 0; r < nreg; ++r) {
    const int L = reg[r].level;
    if (L < 1 || L > 10) return fail(ATHG_ERR_ARG, "refinement level must be in 1..10");
    const double rlo[3] = {reg[r].x1min, reg[r].x2min, reg[r].x3min};
    const double rhi[3] = {reg[r].x1max, reg[r].x2max, reg[r].x3max};
    int64_t a[3], b[3];
    for (int d = 0; d < 3; ++d) {
      if (rlo[d] > rhi[d] || rlo[d] < lo[d] || rhi[d] > hi[d])
        return fail(ATHG_ERR_ARG, "invalid refinement region");
      const int64_t lmax = (int64_t)nrb[d] << L;
      int64_t x = 0;
      for (; x < lmax; ++x)
        if (gen_x(gen_rx(x + 1, lmax), lo[d], hi[d]) > rlo[d]) break;
      int64_t y = x;
      for (; y < lmax; ++y)
        if (gen_x(gen_rx(y + 1, lmax), lo[d], hi[d]) >= rhi[d]) break;
      if (x % 2 == 1) x--;
      if (y % 2 == 0) y++;
      a[d] = x; b[d] = y;
    }
    for (int64_t k = a[2]; k < b[2]; k += 2)
      for (int64_t j = a[1]; j < b[1]; j += 2)
        for (int64_t i = a[0]; i < b[0]; i += 2) {
          const int64_t x[3] = {i, j, k};
          add_block(L, x);
        }
  }
  // 2:1 balance
  for (bool changed = true; changed;) {
    changed = false;
    for (const LocKey& key : leaves) {
      const int L = std::get<0>(key);
      if (L < 2) continue;
      const int64_t x[3] = {std::get<1>(key), std::get<2>(key), std::get<3>(key)};
      for (int o = 0; o < 27 && !changed; ++o) {
        if (o == 13) continue;
        const int off[3] = {o % 3 - 1, (o / 3) % 3 - 1, o / 9 - 1};
        int64_t y[3];
        for (int d = 0; d < 3; ++d) {
          const int64_t n = (int64_t)nrb[d] << L;
          y[d] = ((x[d] + off[d]) % n + n) % n;
        }
        for (int lv = L - 2; lv >= 0; --lv) {
          const int sh = L - lv;
          LocKey an(lv, y[0] >> sh, y[1] >> sh, y[2] >> sh);
          if (leaves.count(an)) { refine(an); changed = true; break; }
        }
      }
      if (changed) break;
    }
  }
  out->clear();
  for (const LocKey& key : leaves) {
    SmrLoc l;
    l.level = std::get<0>(key);
    l.lx[0] = std::get<1>(key); l.lx[1] = std::get<2>(key); l.lx[2] = std::get<3>(key);
    out->push_back(l);
  }
  // level, then lx3, lx2, lx1
  std::sort(out->begin(), out->end(), [](const SmrLoc& p, const SmrLoc& q) {
    return std::make_tuple(p.level, p.lx[2], p.lx[1], p.lx[0]) <
           std::make_tuple(q.level, q.lx[2], q.lx[1], q.lx[0]);
  });
  (void)nmx;
  return ATHG_OK;
}

// Cell widths, cell centres (fine and coarse buffer) and face positions of the leaves
// `loc`, as the reference's Coordinates computes them for its levels
void leaf_coords(const athg_ctx* c, const athg_mesh* m, const std::vector<SmrLoc>& loc,
                 std::vector<double>* dxv, std::vector<double>* xvf, std::vector<double>* xvc,
                 std::vector<double>* faces, int* ncmax, int* nccmax) {
  const Geom& g = c->g;
  const int nmx[3] = {m->nx1, m->nx2, m->nx3};
  const int nbx[3] = {g.nx1, g.nx2, g.nx3};
  const double lo[3] = {m->x1min, m->x2min, m->x3min}, hi[3] = {m->x1max, m->x2max, m->x3max};
  const int ncs[3] = {g.nc1, g.nc2, g.nc3};
  *ncmax = std::max(g.nc1, std::max(g.nc2, g.nc3));
  *nccmax = std::max(nbx[0], std::max(nbx[1], nbx[2])) / 2 + 2 * g.ng;
  const size_t nb = loc.size();
  dxv->assign(nb * 3, 0.0);
  xvf->assign(nb * 3 * *ncmax, 0.0);
  xvc->assign(nb * 3 * *nccmax, 0.0);
  faces->assign(nb * (ncs[0] + ncs[1] + ncs[2] + 3), 0.0);
  size_t off = 0;
  for (size_t b = 0; b < nb; ++b)
    for (int d = 0; d < 3; ++d) {
      smr_axis_coords(nmx[d], nmx[d] / nbx[d], lo[d], hi[d], loc[b].level, loc[b].lx[d], nbx[d],
                      g.ng, &(*dxv)[3 * b + d], &(*xvf)[(b * 3 + d) * *ncmax],
                      &(*xvc)[(b * 3 + d) * *nccmax], &(*faces)[off]);
      off += ncs[d] + 1;
    }
}

// Allocates the pool for the leaves `loc` of a periodic mesh and plans its level
// boundaries; coordinates follow the reference's uniform generator per level
int set_multilevel(athg_ctx* c, const athg_mesh* m, const std::vector<SmrLoc>& loc) {
  for (int d = 0; d < 3; ++d)
    if (!m->periodic[d]) return fail(ATHG_ERR_ARG, "multi-level meshes: periodic boundaries only");
  const Geom& g = c->g;
  const int nmx[3] = {m->nx1, m->nx2, m->nx3};
  const int nbx[3] = {g.nx1, g.nx2, g.nx3};
  int nrb[3];
  for (int d = 0; d < 3; ++d) {
    if (nmx[d] % nbx[d] != 0)
      return fail(ATHG_ERR_ARG, "mesh size must be a multiple of the MeshBlock size");
    nrb[d] = nmx[d] / nbx[d];
  }
  const athg_mesh mcopy = *m;  // m may point at c->mesh
  const int nb = (int)loc.size();
  const int ncs[3] = {g.nc1, g.nc2, g.nc3};
  std::vector<double> dxv, xvf, xvc, faces;
  int ncmax, nccmax;
  leaf_coords(c, &mcopy, loc, &dxv, &xvf, &xvc, &faces, &ncmax, &nccmax);
  c->coords = faces;
  std::vector<athg_block> bl(nb);
  size_t off = 0;
  for (int b = 0; b < nb; ++b) {
    athg_block& B = bl[b];
    B.lx1 = loc[b].lx[0]; B.lx2 = loc[b].lx[1]; B.lx3 = loc[b].lx[2];
    B.level = loc[b].level;
    double* xfs[3];
    for (int d = 0; d < 3; ++d) {
      xfs[d] = &c->coords[off];
      off += ncs[d] + 1;
    }
    B.x1f = xfs[0]; B.x2f = xfs[1]; B.x3f = xfs[2];
    B.dx1 = dxv[3 * b]; B.dx2 = dxv[3 * b + 1]; B.dx3 = dxv[3 * b + 2];
    for (int n = 0; n < 27; ++n) B.neighbor[n] = -1;  // level boundaries use the SMR lists
  }
  int rc = athg_set_blocks(c, nb, bl.data());
  if (rc) return rc;
  c->mesh = mcopy;
  SmrDims d = smr_dims(g.nx1, g.nx2, g.nx3, g.ng);
  std::string err;
  rc = athg::smr_create(&c->smr, d, nrb, loc, dxv, xvf, xvc, c->cfg.magnetic != 0, c->st, &err);
  if (rc) return fail(rc == -1 ? ATHG_ERR_ARG : ATHG_ERR_CUDA, err);
  CK(cudaMalloc(&c->amr_bits, sizeof(unsigned long long) * nb));
  if (c->mixed()) {  // FP64 primitives and bcc of the prolongated ghost cells
    CK(cudaMalloc(&c->smr_w64, sizeof(double) * NHYD * g.ncell * nb));
    CK(cudaMalloc(&c->smr_bcc64, sizeof(double) * 3 * g.ncell * nb));
  }
  if ((int)c->amr_deref.size() != nb) c->amr_deref.assign(nb, 0);
  return ATHG_OK;
}

std::vector<SmrLoc> current_leaves(const athg_ctx* c) {
  std::vector<SmrLoc> l(c->nb);
  for (int b = 0; b < c->nb; ++b) {
    l[b].level = c->blocks[b].level;
    l[b].lx[0] = c->blocks[b].lx1; l[b].lx[1] = c->blocks[b].lx2; l[b].lx[2] = c->blocks[b].lx3;
  }
  return l;
}

template <typename V>
cudaError_t dl(V* host, const double* dev, size_t n, cudaStream_t st) {
  host->resize(n);
  return cudaMemcpyAsync(host->data(), dev, n * sizeof(double), cudaMemcpyDeviceToHost, st);
}
cudaError_t ul(double* dev, const std::vector<double>& host, cudaStream_t st) {
  return cudaMemcpyAsync(dev, host.data(), host.size() * sizeof(double), cudaMemcpyHostToDevice, st);
}

// Mesh::LoadBalancingAndAdaptiveMeshRefinement on one GPU: the criterion on the current
// state, CheckRefinementCondition, UpdateMeshBlockTree and, when the tree changed, the
// new pool (kept blocks, prolongated and restricted ones), its level-boundary plan and
// Initialize(2): ghosts, W(U) and one NewTimeStep from dt_prev. in_cycle adds the main
// loop's NewTimeStep (main.cpp:476-477).
int amr_regrid(athg_ctx* c, bool in_cycle, double dt_prev, int* changed) {
  *changed = 0;
  if (!c->amr || !c->smr) return fail(ATHG_ERR_STATE, "adaptive refinement is not enabled");
  const Geom& g = c->g;
  const int nb = c->nb;
  const SmrDims d = smr_dims(g.nx1, g.nx2, g.nx3, g.ng);
  athg::amr_criterion(d, nb, (const double*)c->w, c->amr_bits, c->st);
  CKL();
  std::vector<unsigned long long> bits(nb);
  CK(cudaMemcpyAsync(bits.data(), c->amr_bits, sizeof(unsigned long long) * nb,
                     cudaMemcpyDeviceToHost, c->st));
  CK(cudaStreamSynchronize(c->st));
  const std::vector<SmrLoc> leaves = current_leaves(c);
  const int nrb[3] = {c->mesh.nx1 / g.nx1, c->mesh.nx2 / g.nx2, c->mesh.nx3 / g.nx3};
  std::vector<int> lv;
  std::string err;
  if (!smr_neighbor_levels(nrb, leaves, &lv, &err)) return fail(ATHG_ERR_STATE, err);
  std::vector<int> flags(nb);
  for (int b = 0; b < nb; ++b) {
    double maxeps;
    std::memcpy(&maxeps, &bits[b], 8);
    flags[b] = amr_flag(maxeps, c->amrc.threshold, c->amrc.deref_fraction, leaves[b].level,
                        c->amrc.max_level, &lv[27 * b], c->amrc.derefine_count, &c->amr_deref[b]);
  }
  std::vector<SmrLoc> nl;
  if (!amr_update_tree(nrb, leaves, flags, &nl)) return ATHG_OK;
  // the old pool on the host
  const bool mhd = c->cfg.magnetic != 0;
  AmrArrays old;
  const int64_t nbl = nb;
  CK(dl(&old.u, c->u, (size_t)(NHYD * g.ncell * nbl), c->st));
  CK(dl(&old.cu, c->smr->cu, (size_t)(5 * d.ccell * nbl), c->st));
  if (mhd) {
    CK(dl(&old.b1, c->b1, (size_t)(g.nf1 * nbl), c->st));
    CK(dl(&old.b2, c->b2, (size_t)(g.nf2 * nbl), c->st));
    CK(dl(&old.b3, c->b3, (size_t)(g.nf3 * nbl), c->st));
    CK(dl(&old.cb1, c->smr->cb1, (size_t)(d.cf1 * nbl), c->st));
    CK(dl(&old.cb2, c->smr->cb2, (size_t)(d.cf2 * nbl), c->st));
    CK(dl(&old.cb3, c->smr->cb3, (size_t)(d.cf3 * nbl), c->st));
  }
  double hs[3];
  CK(cudaMemcpyAsync(hs, c->scal, sizeof(hs), cudaMemcpyDeviceToHost, c->st));
  CK(cudaStreamSynchronize(c->st));
  long long ncyc;
  std::memcpy(&ncyc, &hs[2], 8);
  std::vector<double> old_dx(3 * nbl);
  for (int b = 0; b < nb; ++b) {
    old_dx[3 * b] = c->blocks[b].dx1; old_dx[3 * b + 1] = c->blocks[b].dx2;
    old_dx[3 * b + 2] = c->blocks[b].dx3;
  }
  std::vector<double> dxv, xvf, xvc, faces;
  int ncmax, nccmax;
  leaf_coords(c, &c->mesh, nl, &dxv, &xvf, &xvc, &faces, &ncmax, &nccmax);
  AmrArrays nw;
  std::vector<int> nderef;
  amr_fill(d, mhd, leaves, old, old_dx, c->amr_deref, nl, dxv, xvf, xvc, ncmax, nccmax, &nw,
           &nderef);
  int rc = set_multilevel(c, &c->mesh, nl);
  if (rc) return rc;
  c->amr_deref = nderef;
  CK(ul(c->u, nw.u, c->st));
  CK(ul(c->smr->cu, nw.cu, c->st));
  if (mhd) {
    CK(ul(c->b1, nw.b1, c->st)); CK(ul(c->b2, nw.b2, c->st)); CK(ul(c->b3, nw.b3, c->st));
    CK(ul(c->smr->cb1, nw.cb1, c->st)); CK(ul(c->smr->cb2, nw.cb2, c->st));
    CK(ul(c->smr->cb3, nw.cb3, c->st));
  }
  // Initialize(2): time and ncycle stay, dt restarts from the cycle's dt
  double ts[3] = {hs[0], dt_prev, 0.0};
  std::memcpy(&ts[2], &ncyc, 8);
  CK(cudaMemcpyAsync(c->scal, ts, sizeof(ts), cudaMemcpyHostToDevice, c->st));
  unsigned long long big;
  std::memcpy(&big, &kDblMax, 8);
  CK(cudaMemcpyAsync(c->scal + 3, &big, 8, cudaMemcpyHostToDevice, c->st));
  if ((rc = launch_ghosts(c))) return rc;
  if ((rc = launch_c2p(c))) return rc;
  if ((rc = launch_block_dt(c))) return rc;
  if ((rc = launch_end(c, 0))) return rc;
  if (in_cycle) {
    if ((rc = launch_block_dt(c))) return rc;
    if ((rc = launch_end(c, 0))) return rc;
  }
  CK(cudaStreamSynchronize(c->st));  // the host arrays above go out of scope
  *changed = 1;
  return ATHG_OK;
}

}  // namespace

// =================================================================== C ABI ==========
extern "C" {

const char* athg_last_error(void) { return g_err.c_str(); }

int athg_create(const athg_config* cfg, athg_ctx** out) {
  if (!cfg || !out) return fail(ATHG_ERR_ARG, "null argument");
  *out = nullptr;
  if (cfg->nx1 < 2 || cfg->nx2 < 2 || cfg->nx3 < 2)
    return fail(ATHG_ERR_ARG, "only 3-D MeshBlocks are supported");
  if (cfg->xorder < 1 || cfg->xorder > 3)
    return fail(ATHG_ERR_ARG, "xorder must be 1 (donor cell), 2 (PLM) or 3 (PPM)");
  if (cfg->nghost < 2) return fail(ATHG_ERR_ARG, "nghost must be >= 2");
  // reconstruct/reconstruction.cpp:90-98: PPM needs three ghost layers
  if (cfg->xorder == 3 && cfg->nghost < 3) return fail(ATHG_ERR_ARG, "PPM needs nghost >= 3");
  if (cfg->magnetic &&
      !(cfg->rsolver == ATHG_HLLD || cfg->rsolver == ATHG_HLLE || cfg->rsolver == ATHG_LHLLD))
    return fail(ATHG_ERR_ARG, "MHD needs the HLLD, LHLLD or HLLE solver");
  if (!cfg->magnetic &&
      !(cfg->rsolver == ATHG_HLLC || cfg->rsolver == ATHG_HLLE || cfg->rsolver == ATHG_LHLLC))
    return fail(ATHG_ERR_ARG, "hydro needs the HLLC, LHLLC or HLLE solver");
  if (cfg->precision != ATHG_FP64 && cfg->precision != ATHG_MIXED &&
      cfg->precision != ATHG_DFLOAT)
    return fail(ATHG_ERR_ARG, "precision must be ATHG_FP64, ATHG_MIXED or ATHG_DFLOAT");
  if (cfg->precision == ATHG_DFLOAT &&
      !athg::df_supported(cfg->magnetic, cfg->rsolver, cfg->xorder))
    return fail(ATHG_ERR_ARG, "ATHG_DFLOAT supports donor cell or PLM with HLLC/HLLE (hydro) "
                              "or HLLD/HLLE (MHD)");
  int ndev = 0;
  if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev == 0)
    return fail(ATHG_ERR_CUDA, "no CUDA device available");
  athg_ctx* c = new athg_ctx();
  c->cfg = *cfg;
  if (!make_integrator(cfg->integrator, &c->integ)) {
    delete c;
    return fail(ATHG_ERR_ARG, "unknown integrator");
  }
  if (cudaStreamCreateWithFlags(&c->st, cudaStreamNonBlocking) != cudaSuccess) {
    delete c;
    return fail(ATHG_ERR_CUDA, "cudaStreamCreate failed");
  }
  Geom& g = c->g;
  g.nx1 = cfg->nx1; g.nx2 = cfg->nx2; g.nx3 = cfg->nx3; g.ng = cfg->nghost;
  g.nc1 = g.nx1 + 2 * g.ng; g.nc2 = g.nx2 + 2 * g.ng; g.nc3 = g.nx3 + 2 * g.ng;
  g.is = g.ng; g.ie = g.ng + g.nx1 - 1;
  g.js = g.ng; g.je = g.ng + g.nx2 - 1;
  g.ks = g.ng; g.ke = g.ng + g.nx3 - 1;
  g.ncell = (int64_t)g.nc1 * g.nc2 * g.nc3;
  g.nf1 = (int64_t)g.nc3 * g.nc2 * (g.nc1 + 1);
  g.nf2 = (int64_t)g.nc3 * (g.nc2 + 1) * g.nc1;
  g.nf3 = (int64_t)(g.nc3 + 1) * g.nc2 * g.nc1;
  g.ne = (int64_t)(g.nc3 + 1) * (g.nc2 + 1) * (g.nc1 + 1);
  g.ncmax = std::max(g.nc1, std::max(g.nc2, g.nc3));
  g.dw1 = fastdiv_make((uint32_t)(g.nc1 + 1));
  g.dw2 = fastdiv_make((uint32_t)(g.nc2 + 1));
  g.dgj = fastdiv_make((uint32_t)(g.nc2 + 1 - g.nx2));
  g.dgi = fastdiv_make((uint32_t)(g.nc1 + 1 - g.nx1));
  g.dnx2 = fastdiv_make((uint32_t)g.nx2);
  *out = c;
  return ATHG_OK;
}

int athg_destroy(athg_ctx* c) {
  if (!c) return ATHG_OK;
  free_pool(c);
  if (c->st) cudaStreamDestroy(c->st);
  delete c;
  return ATHG_OK;
}

int athg_set_blocks(athg_ctx* c, int nblocks, const athg_block* blocks) {
  if (!c || nblocks <= 0 || !blocks) return fail(ATHG_ERR_ARG, "bad block list");
  c->outflow = false;  // athg_set_uniform_mesh turns it on for its non-periodic axes
  if (nblocks > 65535) return fail(ATHG_ERR_ARG, "at most 65535 blocks per context");
  for (int b = 0; b < nblocks; ++b) {
    if (!blocks[b].x1f || !blocks[b].x2f || !blocks[b].x3f)
      return fail(ATHG_ERR_ARG, "block coordinates missing");
    for (int n = 0; n < 27; ++n)
      if (blocks[b].neighbor[n] < -1 || blocks[b].neighbor[n] >= nblocks)
        return fail(ATHG_ERR_ARG, "neighbour id out of range");
  }
  free_pool(c);
  const Geom& g0 = c->g;
  c->g.nb = nblocks;
  const Geom& g = c->g;
  (void)g0;
  const int64_t nb = nblocks;
  const size_t tsz = c->mixed() ? sizeof(float) : sizeof(double);
  const bool mhd = c->cfg.magnetic != 0;
  const int NF = mhd ? 8 : 5;
  CK(cudaMalloc(&c->u, sizeof(double) * NHYD * g.ncell * nb));
  CK(cudaMalloc(&c->u1, sizeof(double) * NHYD * g.ncell * nb));
  if (c->dfloat())
    CK(cudaMalloc(&c->wpair_df, sizeof(float2) * (c->cfg.magnetic ? 8 : 5) * g.ncell * nb));
  CK(cudaMalloc(&c->w, tsz * NHYD * g.ncell * nb));
  CK(cudaMalloc(&c->flx[0], tsz * NF * g.nf1 * nb));
  CK(cudaMalloc(&c->flx[1], tsz * NF * g.nf2 * nb));
  CK(cudaMalloc(&c->flx[2], tsz * NF * g.nf3 * nb));
  if (mhd) {
    CK(cudaMalloc(&c->bcc, tsz * 3 * g.ncell * nb));
    CK(cudaMalloc(&c->b1, sizeof(double) * g.nf1 * nb));
    CK(cudaMalloc(&c->b2, sizeof(double) * g.nf2 * nb));
    CK(cudaMalloc(&c->b3, sizeof(double) * g.nf3 * nb));
    CK(cudaMalloc(&c->r1, sizeof(double) * g.nf1 * nb));
    CK(cudaMalloc(&c->r2, sizeof(double) * g.nf2 * nb));
    CK(cudaMalloc(&c->r3, sizeof(double) * g.nf3 * nb));
    CK(cudaMalloc(&c->edge, tsz * 3 * g.ne * nb));
    if (c->mixed()) {
      CK(cudaMalloc(&c->cce, sizeof(float) * 3 * g.ncell * nb));
      CK(cudaMemsetAsync(c->cce, 0, sizeof(float) * 3 * g.ncell * nb, c->st));
      CK(cudaMalloc(&c->bf32[0], sizeof(float) * g.nf1 * nb));
      CK(cudaMalloc(&c->bf32[1], sizeof(float) * g.nf2 * nb));
      CK(cudaMalloc(&c->bf32[2], sizeof(float) * g.nf3 * nb));
      CK(cudaMemsetAsync(c->bf32[0], 0, sizeof(float) * g.nf1 * nb, c->st));
      CK(cudaMemsetAsync(c->bf32[1], 0, sizeof(float) * g.nf2 * nb, c->st));
      CK(cudaMemsetAsync(c->bf32[2], 0, sizeof(float) * g.nf3 * nb, c->st));
    }
    if (c->dfloat()) CK(cudaMalloc(&c->cce_df, sizeof(float2) * 3 * g.ncell * nb));
    CK(cudaMemsetAsync(c->b1, 0, sizeof(double) * g.nf1 * nb, c->st));
    CK(cudaMemsetAsync(c->b2, 0, sizeof(double) * g.nf2 * nb, c->st));
    CK(cudaMemsetAsync(c->b3, 0, sizeof(double) * g.nf3 * nb, c->st));
    CK(cudaMemsetAsync(c->edge, 0, tsz * 3 * g.ne * nb, c->st));
  }
  CK(cudaMemsetAsync(c->u, 0, sizeof(double) * NHYD * g.ncell * nb, c->st));
  CK(cudaMemsetAsync(c->u1, 0, sizeof(double) * NHYD * g.ncell * nb, c->st));
  CK(cudaMalloc(&c->geo, sizeof(BlockGeo) * nb));
  CK(cudaMalloc(&c->coef, tsz * nb * 3 * 2 * g.ncmax));
  CK(cudaMalloc(&c->dxT, tsz * nb * 3));
  CK(cudaMalloc(&c->mg, sizeof(MixedGeo) * nb));
  if (c->mixed()) CK(cudaMalloc(&c->dtf, sizeof(float)));
  CK(cudaMalloc(&c->nbr, sizeof(int) * 27 * nb));
  CK(cudaMalloc(&c->scal, sizeof(double) * 16));
  CK(cudaMemsetAsync(c->scal, 0, sizeof(double) * 16, c->st));
  // host-side per-block tables
  std::vector<BlockGeo> hgeo(nb);
  std::vector<double> hcoef(nb * 3 * 2 * g.ncmax, 0.0);
  std::vector<int> hnbr(27 * nb);
  c->blocks.assign(blocks, blocks + nblocks);
  const int ncs[3] = {g.nc1, g.nc2, g.nc3};
  for (int b = 0; b < nblocks; ++b) {
    const athg_block& B = blocks[b];
    hgeo[b].dx[0] = B.dx1; hgeo[b].dx[1] = B.dx2; hgeo[b].dx[2] = B.dx3;
    const double* xf[3] = {B.x1f, B.x2f, B.x3f};
    for (int d = 0; d < 3; ++d) {
      double* cp = &hcoef[((size_t)b * 3 + d) * 2 * g.ncmax];
      double* cm = cp + g.ncmax;
      const double dx = hgeo[b].dx[d];
      for (int i = 0; i < ncs[d]; ++i) {
        // Cartesian x_v (coordinates/cartesian.cpp:29) and the PLM interface
        // coefficients of reconstruct/plm.cpp:113-119 (x1), :226-227 (x2), :332-333 (x3)
        double xv = 0.5 * (xf[d][i + 1] + xf[d][i]);
        cp[i] = (xf[d][i + 1] - xv) / dx;
        cm[i] = (xv - xf[d][i]) / dx;
      }
    }
    for (int n = 0; n < 27; ++n) hnbr[27 * b + n] = B.neighbor[n];
  }
  CK(cudaMemcpyAsync(c->geo, hgeo.data(), sizeof(BlockGeo) * nb, cudaMemcpyHostToDevice, c->st));
  std::vector<double> hdx(nb * 3);
  for (int b = 0; b < nblocks; ++b)
    for (int d = 0; d < 3; ++d) hdx[b * 3 + d] = hgeo[b].dx[d];
  // Mixed-path widths: blocks of one level whose widths agree to round-off share the
  // first such block's values (uniform meshes), so shared faces and edges carry one weight
  std::vector<MixedGeo> hmg(nb);
  for (int b = 0; b < nblocks; ++b) {
    const double* dx = hgeo[b].dx;
    for (int a = 0; a < b; ++a) {
      if (blocks[a].level != blocks[b].level) continue;
      bool same = true;
      for (int d = 0; d < 3; ++d)
        same = same && std::fabs(hgeo[a].dx[d] - dx[d]) <= 1e-12 * std::fabs(dx[d]);
      if (same) { dx = hgeo[a].dx; break; }
    }
    const double vol = dx[0] * dx[1] * dx[2];
    for (int d = 0; d < 3; ++d) {
      hmg[b].idx[d] = (float)(1.0 / dx[d]);
      hmg[b].dx[d] = (float)dx[d];
      hmg[b].ia[d] = dx[d] / vol;
      const double idx = 1.0 / dx[d];
      hmg[b].idxh[d] = (float)idx;
      hmg[b].idxl[d] = (float)(idx - (double)hmg[b].idxh[d]);
    }
  }
  if (c->mixed()) {
    std::vector<float> fc(hcoef.begin(), hcoef.end()), fdx(hdx.begin(), hdx.end());
    CK(cudaMemcpyAsync(c->coef, fc.data(), sizeof(float) * fc.size(), cudaMemcpyHostToDevice, c->st));
    CK(cudaMemcpyAsync(c->dxT, fdx.data(), sizeof(float) * fdx.size(), cudaMemcpyHostToDevice, c->st));
    CK(cudaStreamSynchronize(c->st));  // the host vectors above go out of scope
  } else {
    CK(cudaMemcpyAsync(c->coef, hcoef.data(), sizeof(double) * hcoef.size(), cudaMemcpyHostToDevice,
                       c->st));
    CK(cudaMemcpyAsync(c->dxT, hdx.data(), sizeof(double) * hdx.size(), cudaMemcpyHostToDevice, c->st));
  }
  CK(cudaMemcpyAsync(c->mg, hmg.data(), sizeof(MixedGeo) * nb, cudaMemcpyHostToDevice, c->st));
  CK(cudaMemcpyAsync(c->nbr, hnbr.data(), sizeof(int) * hnbr.size(), cudaMemcpyHostToDevice,
                     c->st));
  double hs[16] = {0};
  hs[1] = kDblMax;
  unsigned long long big;
  std::memcpy(&big, &kDblMax, 8);
  std::memcpy(&hs[3], &big, 8);
  CK(cudaMemcpyAsync(c->scal, hs, sizeof(hs), cudaMemcpyHostToDevice, c->st));
  CK(cudaStreamSynchronize(c->st));
  // the host copies of the coordinate pointers are not kept
  for (auto& B : c->blocks) B.x1f = B.x2f = B.x3f = nullptr;
  c->nb = nblocks;
  return ATHG_OK;
}

int athg_set_uniform_mesh(athg_ctx* c, const athg_mesh* m) {
  if (!c || !m) return fail(ATHG_ERR_ARG, "null argument");
  const Geom& g = c->g;
  const int nmx[3] = {m->nx1, m->nx2, m->nx3};
  const int nbx[3] = {g.nx1, g.nx2, g.nx3};
  const double lo[3] = {m->x1min, m->x2min, m->x3min}, hi[3] = {m->x1max, m->x2max, m->x3max};
  int nrb[3];
  for (int d = 0; d < 3; ++d) {
    if (nmx[d] % nbx[d] != 0)
      return fail(ATHG_ERR_ARG, "mesh size must be a multiple of the MeshBlock size");
    if (m->periodic[d] != 0 && m->periodic[d] != 1)
      return fail(ATHG_ERR_ARG, "periodic[d] must be 1 (periodic) or 0 (outflow)");
    if (!m->periodic[d] && c->mixed())
      return fail(ATHG_ERR_ARG, "outflow boundaries run on the FP64 and double-float paths "
                                "(precision ATHG_FP64 or ATHG_DFLOAT)");
    nrb[d] = nmx[d] / nbx[d];
  }
  const int nblocks = nrb[0] * nrb[1] * nrb[2];
  std::vector<athg_block> bl(nblocks);
  const int ncs[3] = {g.nc1, g.nc2, g.nc3};
  c->coords.assign((size_t)nblocks * (ncs[0] + ncs[1] + ncs[2] + 3), 0.0);
  size_t off = 0;
  for (int b3 = 0; b3 < nrb[2]; ++b3)
    for (int b2 = 0; b2 < nrb[1]; ++b2)
      for (int b1 = 0; b1 < nrb[0]; ++b1) {
        const int id = (b3 * nrb[1] + b2) * nrb[0] + b1;
        athg_block& B = bl[id];
        const int lx[3] = {b1, b2, b3};
        B.lx1 = b1; B.lx2 = b2; B.lx3 = b3; B.level = 0;
        double* xfs[3];
        double dxs[3];
        for (int d = 0; d < 3; ++d) {
          // block_size (mesh/mesh.cpp:1675-1690): exact mesh bounds at the edges
          double bmin = (lx[d] == 0) ? lo[d] : gen_x(gen_rx(lx[d], nrb[d]), lo[d], hi[d]);
          double bmax = (lx[d] == nrb[d] - 1) ? hi[d]
                                               : gen_x(gen_rx(lx[d] + 1, nrb[d]), lo[d], hi[d]);
          // face positions (coordinates/coordinates.cpp:127-145, uniform branch)
          const int il = g.ng, iu = g.ng + nbx[d] - 1;
          double* xf = &c->coords[off];
          off += ncs[d] + 1;
          dxs[d] = (bmax - bmin) / (iu - il + 1);
          for (int i = il - g.ng; i <= iu + g.ng + 1; ++i) {
            int64_t noff = (int64_t)(i - il) + (int64_t)lx[d] * nbx[d];
            xf[i] = gen_x(gen_rx(noff, nmx[d]), lo[d], hi[d]);
          }
          xf[il] = bmin;
          xf[iu + 1] = bmax;
          xfs[d] = xf;
        }
        B.x1f = xfs[0]; B.x2f = xfs[1]; B.x3f = xfs[2];
        B.dx1 = dxs[0]; B.dx2 = dxs[1]; B.dx3 = dxs[2];
        for (int o3 = -1; o3 <= 1; ++o3)
          for (int o2 = -1; o2 <= 1; ++o2)
            for (int o1 = -1; o1 <= 1; ++o1) {
              int n[3] = {b1 + o1, b2 + o2, b3 + o3};
              bool ok = true;
              for (int d = 0; d < 3; ++d) {
                if (n[d] < 0 || n[d] >= nrb[d]) {
                  if (m->periodic[d]) n[d] = (n[d] + nrb[d]) % nrb[d];
                  else ok = false;
                }
              }
              B.neighbor[(o3 + 1) * 9 + (o2 + 1) * 3 + (o1 + 1)] =
                  ok ? (n[2] * nrb[1] + n[1]) * nrb[0] + n[0] : -1;
            }
      }
  const athg_mesh mcopy = *m;
  int rc = athg_set_blocks(c, nblocks, bl.data());
  if (!rc) {
    c->mesh = mcopy;
    c->outflow = !(m->periodic[0] && m->periodic[1] && m->periodic[2]);
  }
  return rc;
}

int athg_set_refined_mesh(athg_ctx* c, const athg_mesh* m, int nregions,
                          const athg_region* regions) {
  if (!c || !m || nregions < 0 || (nregions > 0 && !regions))
    return fail(ATHG_ERR_ARG, "null argument");
  const Geom& g = c->g;
  const int nmx[3] = {m->nx1, m->nx2, m->nx3};
  const int nbx[3] = {g.nx1, g.nx2, g.nx3};
  const double lo[3] = {m->x1min, m->x2min, m->x3min}, hi[3] = {m->x1max, m->x2max, m->x3max};
  int nrb[3];
  for (int d = 0; d < 3; ++d) {
    if (nbx[d] <= 0 || nmx[d] % nbx[d] != 0)
      return fail(ATHG_ERR_ARG, "mesh size must be a multiple of the MeshBlock size");
    nrb[d] = nmx[d] / nbx[d];
  }
  std::vector<SmrLoc> loc;
  int rc = refined_leaves(nmx, nrb, lo, hi, nregions, regions, &loc);
  if (rc) return rc;
  return set_multilevel(c, m, loc);
}

int athg_set_multilevel_blocks(athg_ctx* c, const athg_mesh* m, int nblocks,
                               const int64_t* locs) {
  if (!c || !m || nblocks <= 0 || !locs) return fail(ATHG_ERR_ARG, "null argument");
  std::vector<SmrLoc> loc(nblocks);
  for (int b = 0; b < nblocks; ++b) {
    loc[b].level = (int)locs[4 * b];
    for (int d = 0; d < 3; ++d) loc[b].lx[d] = locs[4 * b + 1 + d];
    if (loc[b].level < 0 || loc[b].level > 10) return fail(ATHG_ERR_ARG, "block level out of range");
  }
  return set_multilevel(c, m, loc);
}

int athg_amr_enable(athg_ctx* c, const athg_amr_config* cfg) {
  int rc = need_pool(c);
  if (rc) return rc;
  if (!cfg) return fail(ATHG_ERR_ARG, "null argument");
  if (c->mixed())
    return fail(ATHG_ERR_ARG, "adaptive refinement runs on the FP64 path (precision ATHG_FP64)");
  if (cfg->max_level < 0 || cfg->max_level > 10 || cfg->derefine_count < 1 ||
      !(cfg->threshold > 0.0))
    return fail(ATHG_ERR_ARG, "invalid adaptive refinement parameters");
  if (!c->smr) {  // a uniform mesh becomes a one-level multi-level mesh, state kept
    const Geom& g = c->g;
    const bool mhd = c->cfg.magnetic != 0;
    const int64_t nb = c->nb;
    std::vector<double> u, b1, b2, b3;
    CK(dl(&u, c->u, (size_t)(NHYD * g.ncell * nb), c->st));
    if (mhd) {
      CK(dl(&b1, c->b1, (size_t)(g.nf1 * nb), c->st));
      CK(dl(&b2, c->b2, (size_t)(g.nf2 * nb), c->st));
      CK(dl(&b3, c->b3, (size_t)(g.nf3 * nb), c->st));
    }
    CK(cudaStreamSynchronize(c->st));
    const athg_mesh m = c->mesh;
    rc = set_multilevel(c, &m, current_leaves(c));
    if (rc) return rc;
    CK(ul(c->u, u, c->st));
    if (mhd) { CK(ul(c->b1, b1, c->st)); CK(ul(c->b2, b2, c->st)); CK(ul(c->b3, b3, c->st)); }
    CK(cudaStreamSynchronize(c->st));
  }
  c->amr = true;
  c->amrc = *cfg;
  c->amr_deref.assign(c->nb, 0);
  return ATHG_OK;
}

int athg_amr_regrid(athg_ctx* c, int* changed) {
  int rc = need_pool(c);
  if (rc) return rc;
  if (!changed) return fail(ATHG_ERR_ARG, "null argument");
  double dt;
  CK(cudaMemcpyAsync(&dt, c->scal + 1, 8, cudaMemcpyDeviceToHost, c->st));
  CK(cudaStreamSynchronize(c->st));
  return amr_regrid(c, false, dt, changed);
}

int athg_smr_stats(athg_ctx* c, int64_t* out8) {
  if (!c || !out8) return fail(ATHG_ERR_ARG, "null argument");
  for (int i = 0; i < 8; ++i) out8[i] = 0;
  if (!c->smr) return ATHG_OK;
  const athg::SmrDevice* s = c->smr;
  out8[0] = s->nxfer; out8[1] = s->npre; out8[2] = s->nflux; out8[3] = s->nemf;
  out8[4] = s->nc2p; out8[5] = s->npcc; out8[6] = s->npint; out8[7] = s->npfine;
  return ATHG_OK;
}

int athg_num_blocks(const athg_ctx* c, int* nblocks) {
  if (!c || !nblocks) return fail(ATHG_ERR_ARG, "null argument");
  *nblocks = c->nb;
  return ATHG_OK;
}

int athg_block_location(const athg_ctx* c, int block, int64_t* out) {
  if (!c || !out || block < 0 || block >= c->nb) return fail(ATHG_ERR_ARG, "bad block");
  const athg_block& B = c->blocks[block];
  out[0] = B.lx1; out[1] = B.lx2; out[2] = B.lx3; out[3] = B.level;
  return ATHG_OK;
}

int athg_var_size(const athg_ctx* c, int var, size_t* count) {
  if (!c || !count) return fail(ATHG_ERR_ARG, "null argument");
  const Geom& g = c->g;
  switch (var) {
    case ATHG_VAR_CONS: case ATHG_VAR_PRIM: *count = (size_t)NHYD * g.ncell; break;
    case ATHG_VAR_B1F: *count = (size_t)g.nf1; break;
    case ATHG_VAR_B2F: *count = (size_t)g.nf2; break;
    case ATHG_VAR_B3F: *count = (size_t)g.nf3; break;
    case ATHG_VAR_BCC: *count = (size_t)3 * g.ncell; break;
    case ATHG_VAR_PHI: *count = (size_t)g.ncell; break;
    default: return fail(ATHG_ERR_ARG, "unknown variable");
  }
  return ATHG_OK;
}

namespace {
// device array of var and whether it is stored in the flux precision (float when mixed)
int var_ptr(athg_ctx* c, int var, void** p, bool* narrow) {
  *narrow = false;
  switch (var) {
    case ATHG_VAR_CONS: *p = c->u; return ATHG_OK;
    case ATHG_VAR_B1F: *p = c->b1; break;
    case ATHG_VAR_B2F: *p = c->b2; break;
    case ATHG_VAR_B3F: *p = c->b3; break;
    case ATHG_VAR_PRIM: *p = c->w; *narrow = c->mixed(); return ATHG_OK;
    case ATHG_VAR_BCC: *p = c->bcc; *narrow = c->mixed(); break;
    case ATHG_VAR_PHI:
      if (!c->phi) return fail(ATHG_ERR_ARG, "no self-gravity attached");
      *p = c->phi;
      return ATHG_OK;
    default: return fail(ATHG_ERR_ARG, "variable not available");
  }
  if (!c->cfg.magnetic) return fail(ATHG_ERR_ARG, "no magnetic field in a hydro context");
  return ATHG_OK;
}
}  // namespace

int athg_upload(athg_ctx* c, int block, int var, const double* host, size_t count) {
  int rc = need_pool(c);
  if (rc) return rc;
  size_t per;
  if ((rc = athg_var_size(c, var, &per))) return rc;
  void* d;
  bool narrow;
  if ((rc = var_ptr(c, var, &d, &narrow))) return rc;
  if (narrow) return fail(ATHG_ERR_ARG, "derived variables cannot be uploaded");
  if (block < -1 || block >= c->nb) return fail(ATHG_ERR_ARG, "bad block index");
  size_t n = (block < 0) ? per * c->nb : per;
  if (!host || count != n) return fail(ATHG_ERR_ARG, "host buffer size mismatch");
  double* dst = (double*)d + (block < 0 ? 0 : per * block);
  CK(cudaMemcpyAsync(dst, host, n * sizeof(double), cudaMemcpyHostToDevice, c->st));
  CK(cudaStreamSynchronize(c->st));
  return ATHG_OK;
}

int athg_download(athg_ctx* c, int block, int var, double* host, size_t count) {
  int rc = need_pool(c);
  if (rc) return rc;
  if (var == ATHG_VAR_CONS || var == ATHG_VAR_B1F || var == ATHG_VAR_B2F || var == ATHG_VAR_B3F)
    if ((rc = refresh_ghosts(c))) return rc;
  size_t per;
  if ((rc = athg_var_size(c, var, &per))) return rc;
  void* d;
  bool narrow;
  if ((rc = var_ptr(c, var, &d, &narrow))) return rc;
  if (block < -1 || block >= c->nb) return fail(ATHG_ERR_ARG, "bad block index");
  size_t n = (block < 0) ? per * c->nb : per;
  if (!host || count != n) return fail(ATHG_ERR_ARG, "host buffer size mismatch");
  size_t off = (block < 0 ? 0 : per * block);
  if (!narrow) {
    CK(cudaMemcpyAsync(host, (double*)d + off, n * sizeof(double), cudaMemcpyDeviceToHost,
                       c->st));
    CK(cudaStreamSynchronize(c->st));
  } else {
    std::vector<float> tmp(n);
    CK(cudaMemcpyAsync(tmp.data(), (float*)d + off, n * sizeof(float), cudaMemcpyDeviceToHost,
                       c->st));
    CK(cudaStreamSynchronize(c->st));
    for (size_t q = 0; q < n; ++q) host[q] = tmp[q];
  }
  return ATHG_OK;
}

int athg_initialize(athg_ctx* c) {
  int rc = need_pool(c);
  if (rc) return rc;
  double hs[4];
  hs[0] = 0.0; hs[1] = kDblMax; hs[2] = 0.0;
  unsigned long long big;
  std::memcpy(&big, &kDblMax, 8);
  std::memcpy(&hs[3], &big, 8);
  CK(cudaMemcpyAsync(c->scal, hs, sizeof(hs), cudaMemcpyHostToDevice, c->st));
  // the first perturbation of decaying or impulsive turbulence (mesh/mesh.cpp:1383-1384)
  if (c->turb && athg::turb_flag(c->turb) <= 2 && (rc = turb_drive(c))) return rc;
  if (has_gravity(c) && (rc = gravity_solve(c, c->u))) return rc;  // mesh/mesh.cpp:1398-1402
  if ((rc = launch_ghosts(c))) return rc;
  c->ghosts_stale = false;
  if ((rc = launch_c2p(c))) return rc;
  if ((rc = launch_block_dt(c))) return rc;
  if ((rc = launch_end(c, 0))) return rc;
  CK(cudaStreamSynchronize(c->st));
  return ATHG_OK;
}

int athg_resume(athg_ctx* c) {
  int rc = need_pool(c);
  if (rc) return rc;
  // Mesh::Initialize on a restart (res_flag = 1): time, dt and ncycle stay as read from
  // the restart file (athg_set_time); ghosts, W(U), then NewTimeStep from the stored dt
  unsigned long long big;
  std::memcpy(&big, &kDblMax, 8);
  CK(cudaMemcpyAsync(c->scal + 3, &big, 8, cudaMemcpyHostToDevice, c->st));
  if (has_gravity(c) && (rc = gravity_solve(c, c->u))) return rc;
  if ((rc = launch_ghosts(c))) return rc;
  c->ghosts_stale = false;
  if ((rc = launch_c2p(c))) return rc;
  if ((rc = launch_block_dt(c))) return rc;
  if ((rc = launch_end(c, 0))) return rc;
  CK(cudaStreamSynchronize(c->st));
  return ATHG_OK;
}

int athg_stage(athg_ctx* c, int stage) {
  int rc = need_pool(c);
  if (rc) return rc;
  if (stage < 1 || stage > c->integ.nstages) return fail(ATHG_ERR_ARG, "stage out of range");
  return do_stage(c, stage);
}

int athg_end_cycle(athg_ctx* c) {
  int rc = need_pool(c);
  if (rc) return rc;
  if ((rc = launch_end(c, 1))) return rc;
  if (fused(c)) swap_state(c);
  return ATHG_OK;
}

int athg_cycles(athg_ctx* c, int n) {
  int rc = need_pool(c);
  if (rc) return rc;
  if (n <= 0) return ATHG_OK;
  if (c->turb && athg::turb_flag(c->turb) > 1) {
    // driven turbulence: Driving before every cycle (main.cpp:457), random numbers on the host
    for (int q = 0; q < n; ++q) {
      if ((rc = turb_drive(c))) return rc;
      if (!captured(c)) {
        if ((rc = run_cycle_direct(c))) return rc;
      } else {
        if ((rc = build_graph(c))) return rc;
        if ((rc = run_cycle_graph(c))) return rc;
      }
    }
    return ATHG_OK;
  }
  if (!captured(c)) {
    // the solve iterates to a threshold or sets up multipole moments on the host, or
    // runs cuFFT
    for (int q = 0; q < n; ++q)
      if ((rc = run_cycle_direct(c))) return rc;
    return ATHG_OK;
  }
  if (c->amr) {  // the refinement check after every cycle (main.cpp:470-477)
    for (int q = 0; q < n; ++q) {
      double dt;
      CK(cudaMemcpyAsync(&dt, c->scal + 1, 8, cudaMemcpyDeviceToHost, c->st));
      CK(cudaStreamSynchronize(c->st));
      if ((rc = build_graph(c))) return rc;
      if ((rc = run_cycle_graph(c))) return rc;
      int changed;
      if ((rc = amr_regrid(c, true, dt, &changed))) return rc;
    }
    return ATHG_OK;
  }
  if ((rc = build_graph(c))) return rc;
  for (int q = 0; q < n; ++q)
    if ((rc = run_cycle_graph(c))) return rc;
  return ATHG_OK;
}

int athg_cycle_timing(athg_ctx* c, int max, double* ms, int* n, char* names,
                      size_t names_size) {
  int rc = need_pool(c);
  if (rc) return rc;
  if (!ms || !n || max <= 0) return fail(ATHG_ERR_ARG, "null argument");
  if ((rc = autotune(c))) return rc;
  std::vector<std::pair<std::string, cudaEvent_t>> ev;
  c->tev = &ev;
  mark(c, 0, "start");
  rc = do_cycle(c);
  c->tev = nullptr;
  if (!rc && fused(c)) {  // as run_cycle_graph: the new state is in the other buffer
    swap_state(c);
    c->ghosts_stale = true;
  }
  cudaError_t e = ev.empty() ? cudaSuccess : cudaEventSynchronize(ev.back().second);
  std::string all;
  int k = 0;
  for (size_t q = 1; q < ev.size() && e == cudaSuccess; ++q) {
    float t = 0.0f;
    e = cudaEventElapsedTime(&t, ev[q - 1].second, ev[q].second);
    if (k < max) {
      ms[k++] = t;
      all += ev[q].first + "\n";
    }
  }
  for (auto& x : ev) cudaEventDestroy(x.second);
  if (rc) return rc;
  if (e != cudaSuccess) return fail(ATHG_ERR_CUDA, std::string("timing: ") + cudaGetErrorString(e));
  *n = k;
  if (names && names_size > 0) {
    const size_t m = std::min(all.size(), names_size - 1);
    std::memcpy(names, all.data(), m);
    names[m] = 0;
  }
  return ATHG_OK;
}

int athg_launches_per_cycle(athg_ctx* c, int* n) {
  int rc = need_pool(c);
  if (rc) return rc;
  if (!n) return fail(ATHG_ERR_ARG, "null argument");
  if (!captured(c))
    return fail(ATHG_ERR_STATE, "cycles with this gravity solver are not captured as a graph");
  if ((rc = build_graph(c))) return rc;
  *n = c->launches_per_cycle;
  return ATHG_OK;
}

int athg_attach_gravity(athg_ctx* c, athg_mg* mg, double four_pi_G) {
  int rc = need_pool(c);
  if (rc) return rc;
  // drop any captured cycle: the stage sequence changes
  drop_graphs(c);
  if ((rc = refresh_ghosts(c))) return rc;
  if (c->grav) athg::mg_bind_stream(c->grav, nullptr);
  c->grav = nullptr;
  athg::fftgrav_destroy(c->fgrav);
  c->fgrav = nullptr;
  if (!mg) return ATHG_OK;
  if (c->smr) return fail(ATHG_ERR_ARG, "self-gravity on a multi-level mesh is not supported");
  double *um, *src;
  int n;
  if ((rc = athg::mg_finest(mg, &um, &src, &n))) return rc;
  // one uniform level tiling the solver's n^3 root grid
  if ((rc = tile_blocks(c, n, n, n))) return rc;
  CK(cudaMemsetAsync(c->phi, 0, sizeof(double) * c->g.ncell * c->nb, c->st));
  if (c->phi2) CK(cudaMemsetAsync(c->phi2, 0, sizeof(float2) * c->g.ncell * c->nb, c->st));
  if ((rc = athg::mg_bind_stream(mg, c->st))) return rc;
  c->grav = mg;
  c->four_pi_G = four_pi_G;
  return ATHG_OK;
}

int athg_attach_fft_gravity(athg_ctx* c, const athg_mesh* mesh, double four_pi_G) {
  int rc = need_pool(c);
  if (rc) return rc;
  drop_graphs(c);
  if ((rc = refresh_ghosts(c))) return rc;
  if (c->grav) athg::mg_bind_stream(c->grav, nullptr);
  c->grav = nullptr;
  athg::fftgrav_destroy(c->fgrav);
  c->fgrav = nullptr;
  if (four_pi_G == 0.0) return ATHG_OK;
  if (!mesh) return fail(ATHG_ERR_ARG, "null argument");
  if ((rc = tile_blocks(c, mesh->nx1, mesh->nx2, mesh->nx3))) return rc;
  CK(cudaMemsetAsync(c->phi, 0, sizeof(double) * c->g.ncell * c->nb, c->st));
  if (c->phi2) CK(cudaMemsetAsync(c->phi2, 0, sizeof(float2) * c->g.ncell * c->nb, c->st));
  athg::FftMesh fm{{mesh->nx1, mesh->nx2, mesh->nx3},
                   {mesh->x1max - mesh->x1min, mesh->x2max - mesh->x2min, mesh->x3max - mesh->x3min}};
  std::string err;
  if (athg::fftgrav_create(fm, four_pi_G, &c->fgrav, &err)) return fail(ATHG_ERR_CUDA, err);
  c->four_pi_G = four_pi_G;
  return ATHG_OK;
}

int athg_turb_attach(athg_ctx* c, const athg_mesh* mesh, const athg_turb_config* cfg) {
  int rc = need_pool(c);
  if (rc) return rc;
  athg::turb_destroy(c->turb);
  c->turb = nullptr;
  if (!cfg) return ATHG_OK;
  if (!mesh) return fail(ATHG_ERR_ARG, "null argument");
  if ((rc = tile_blocks(c, mesh->nx1, mesh->nx2, mesh->nx3))) return rc;
  double t0;
  CK(cudaMemcpyAsync(&t0, c->scal, 8, cudaMemcpyDeviceToHost, c->st));
  CK(cudaStreamSynchronize(c->st));
  athg::FftMesh fm{{mesh->nx1, mesh->nx2, mesh->nx3},
                   {mesh->x1max - mesh->x1min, mesh->x2max - mesh->x2min, mesh->x3max - mesh->x3min}};
  std::string err;
  if ((rc = athg::turb_create(fm, *cfg, t0, &c->turb, &err)))
    return fail(rc > 0 ? ATHG_ERR_ARG : ATHG_ERR_CUDA, err);
  return ATHG_OK;
}

int athg_turb_drive(athg_ctx* c) {
  int rc = need_pool(c);
  if (rc) return rc;
  if (!c->turb) return fail(ATHG_ERR_STATE, "no turbulence driver attached");
  return turb_drive(c);
}

int athg_get_time(athg_ctx* c, double* time, double* dt, int64_t* ncycle) {
  int rc = need_pool(c);
  if (rc) return rc;
  double hs[3];
  CK(cudaMemcpyAsync(hs, c->scal, sizeof(hs), cudaMemcpyDeviceToHost, c->st));
  CK(cudaStreamSynchronize(c->st));
  if ((rc = device_errors(c))) return rc;
  if (time) *time = hs[0];
  if (dt) *dt = hs[1];
  long long nc;
  std::memcpy(&nc, &hs[2], 8);
  if (ncycle) *ncycle = nc;
  return ATHG_OK;
}

int athg_set_time(athg_ctx* c, double time, double dt, int64_t ncycle) {
  int rc = need_pool(c);
  if (rc) return rc;
  double hs[3];
  hs[0] = time; hs[1] = dt;
  long long nc = ncycle;
  std::memcpy(&hs[2], &nc, 8);
  CK(cudaMemcpyAsync(c->scal, hs, sizeof(hs), cudaMemcpyHostToDevice, c->st));
  float df = (float)dt;
  if (c->dtf) CK(cudaMemcpyAsync(c->dtf, &df, sizeof(float), cudaMemcpyHostToDevice, c->st));
  CK(cudaStreamSynchronize(c->st));
  return ATHG_OK;
}

int athg_synchronize(athg_ctx* c) {
  if (!c) return fail(ATHG_ERR_ARG, "null context");
  CK(cudaStreamSynchronize(c->st));
  return c->nb > 0 ? device_errors(c) : ATHG_OK;
}

int athg_stream(athg_ctx* c, void** stream) {
  if (!c || !stream) return fail(ATHG_ERR_ARG, "null argument");
  *stream = (void*)c->st;
  return ATHG_OK;
}

int athg_calculate_fluxes(athg_ctx* c, int order) {
  int rc = need_pool(c);
  if (rc) return rc;
  if ((rc = leave_fused(c))) return rc;
  if (order < 1 || order > 3) return fail(ATHG_ERR_ARG, "order must be 1, 2 or 3");
  if (order == 3 && c->g.ng < 3) return fail(ATHG_ERR_ARG, "PPM needs nghost >= 3");
  return launch_fluxes(c, order);
}

int athg_compute_corner_e(athg_ctx* c) {
  int rc = need_pool(c);
  if (rc) return rc;
  if ((rc = leave_fused(c))) return rc;
  return launch_corner(c);
}

int athg_integrate(athg_ctx* c, int stage) {
  int rc = need_pool(c);
  if (rc) return rc;
  if ((rc = leave_fused(c))) return rc;
  if (stage < 1 || stage > c->integ.nstages) return fail(ATHG_ERR_ARG, "stage out of range");
  return launch_update(c, stage - 1);
}

int athg_exchange_ghosts(athg_ctx* c) {
  int rc = need_pool(c);
  if (rc) return rc;
  if ((rc = leave_fused(c))) return rc;
  return launch_ghosts(c);
}

int athg_conserved_to_primitive(athg_ctx* c) {
  int rc = need_pool(c);
  if (rc) return rc;
  if ((rc = leave_fused(c))) return rc;
  return launch_c2p(c);
}

int athg_new_block_dt(athg_ctx* c, double* dt_out) {
  int rc = need_pool(c);
  if (rc) return rc;
  unsigned long long big;
  std::memcpy(&big, &kDblMax, 8);
  CK(cudaMemcpyAsync(c->scal + 3, &big, 8, cudaMemcpyHostToDevice, c->st));
  if ((rc = launch_block_dt(c))) return rc;
  unsigned long long bits;
  CK(cudaMemcpyAsync(&bits, c->scal + 3, 8, cudaMemcpyDeviceToHost, c->st));
  CK(cudaMemcpyAsync(c->scal + 3, &big, 8, cudaMemcpyHostToDevice, c->st));
  CK(cudaStreamSynchronize(c->st));
  double v;
  std::memcpy(&v, &bits, 8);
  if (dt_out) *dt_out = v * c->cfg.cfl_number;
  return ATHG_OK;
}

int athg_max_div_b(athg_ctx* c, double* out) {
  int rc = need_pool(c);
  if (rc) return rc;
  if (!c->cfg.magnetic) return fail(ATHG_ERR_ARG, "no magnetic field in a hydro context");
  const Geom& g = c->g;
  CK(cudaMemsetAsync(c->scal + 9, 0, 8, c->st));
  dim3 grid((unsigned)((g.nx1 * g.nx2 + 255) / 256), (unsigned)g.nx3, (unsigned)c->nb);
  k_divb<<<grid, 256, 0, c->st>>>(g, c->b1, c->b2, c->b3, c->geo,
                                  (unsigned long long*)(c->scal + 9));
  CKL();
  double v;
  CK(cudaMemcpyAsync(&v, c->scal + 9, 8, cudaMemcpyDeviceToHost, c->st));
  CK(cudaStreamSynchronize(c->st));
  *out = v;
  return ATHG_OK;
}

int athg_sum_conserved(athg_ctx* c, double* out5) {
  int rc = need_pool(c);
  if (rc) return rc;
  const Geom& g = c->g;
  CK(cudaMemsetAsync(c->scal + 4, 0, 5 * 8, c->st));
  dim3 grid((unsigned)((g.nx1 * g.nx2 + 255) / 256), (unsigned)g.nx3, (unsigned)c->nb);
  k_sum_cons<<<grid, 256, 0, c->st>>>(g, c->u, c->geo, c->scal + 4);
  CKL();
  CK(cudaMemcpyAsync(out5, c->scal + 4, 5 * 8, cudaMemcpyDeviceToHost, c->st));
  CK(cudaStreamSynchronize(c->st));
  return ATHG_OK;
}

int athg_get_tuning(athg_ctx* c, int* out3) {
  int rc = need_pool(c);
  if (rc) return rc;
  if (!out3) return fail(ATHG_ERR_ARG, "null argument");
  const FluxTune& t = c->tune[c->cfg.xorder];
  out3[0] = t.x1_tpb; out3[1] = t.march_tpb; out3[2] = t.seg;
  return ATHG_OK;
}

int athg_set_tuning(athg_ctx* c, const int* in3) {
  int rc = need_pool(c);
  if (rc) return rc;
  if (!in3) return fail(ATHG_ERR_ARG, "null argument");
  if ((in3[0] != 64 && in3[0] != 128) || (in3[1] != 64 && in3[1] != 128) || in3[2] < 0)
    return fail(ATHG_ERR_ARG, "threads per block must be 64 or 128, segment length >= 0");
  drop_graphs(c);  // captured cycles hold the old launch shape
  for (FluxTune& t : c->tune) {
    t.x1_tpb = in3[0]; t.march_tpb = in3[1]; t.seg = in3[2];
  }
  c->tuned = true;
  return ATHG_OK;
}

int athg_set_stage_kernel(athg_ctx* c, int single, int nseg) {
  int rc = need_pool(c);
  if (rc) return rc;
  if (nseg < 0 || (nseg > 0 && !athg::single_pass_fits(c->g, nseg)))
    return fail(ATHG_ERR_ARG, "k-segments must divide the block's nx3 (0: autotuned)");
  drop_graphs(c);  // captured cycles hold the old stage sequence
  c->sp_on = (single != 0);
  if (nseg > 0) { c->sp_nseg = nseg; c->sp_tuned = true; }
  else c->sp_tuned = false;
  return ATHG_OK;
}

int athg_get_stage_kernel(athg_ctx* c, int* single, int* nseg) {
  int rc = need_pool(c);
  if (rc) return rc;
  if (!single || !nseg) return fail(ATHG_ERR_ARG, "null argument");
  *single = single_pass(c) ? 1 : 0;
  *nseg = c->sp_nseg;
  return ATHG_OK;
}

int athg_history(athg_ctx* c, double* out, int* count) {
  int rc = need_pool(c);
  if (rc) return rc;
  if (!out || !count) return fail(ATHG_ERR_ARG, "null argument");
  if ((rc = refresh_ghosts(c))) return rc;
  const Geom& g = c->g;
  dim3 grid((unsigned)((g.nx1 * g.nx2 + 255) / 256), (unsigned)g.nx3, (unsigned)c->nb);
  const size_t np = (size_t)grid.x * grid.y * grid.z;
  double* part = nullptr;
  CK(cudaMallocAsync(&part, np * kHist * sizeof(double), c->st));
  k_history<<<grid, 256, 0, c->st>>>(g, c->u, c->b1, c->b2, c->b3, has_gravity(c) ? c->phi : nullptr,
                                     c->geo, c->cfg.magnetic, part);
  cudaError_t e = cudaGetLastError();
  std::vector<double> h(np * kHist);
  if (e == cudaSuccess)
    e = cudaMemcpyAsync(h.data(), part, h.size() * sizeof(double), cudaMemcpyDeviceToHost, c->st);
  cudaFreeAsync(part, c->st);
  if (e == cudaSuccess) e = cudaStreamSynchronize(c->st);
  if (e != cudaSuccess) return fail(ATHG_ERR_CUDA, std::string("history: ") + cudaGetErrorString(e));
  for (int n = 0; n < kHist; ++n) out[n] = 0.0;
  for (size_t q = 0; q < np; ++q)
    for (int n = 0; n < kHist; ++n) out[n] += h[q * kHist + n];
  *count = kHist;
  return ATHG_OK;
}

}  // extern "C"
