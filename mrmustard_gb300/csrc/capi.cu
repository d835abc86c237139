// C ABI of the GB300 Hermite library: argument checks, workspace layout,
// ragged-batch planning and kernel launches.  See include/mm_gb300.h.
#include <algorithm>
#include <cmath>
#include <atomic>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <mutex>
#include <new>
#include <vector>

#include "kernels.cuh"

using namespace mm;

namespace {

thread_local char g_last_cuda_error[256] = "";
std::atomic<int64_t> g_launches{0};

constexpr int64_t kGridMinAmps = 4096;     // single instances at least this large use the whole grid (default)
constexpr int kGridBlock = 512;            // threads per CTA of the cooperative stable kernel
constexpr int kFlowBlock = 256;            // dataflow forward: threads per CTA
constexpr int kFlowPerSm = 2;              // dataflow forward: CTAs per SM (capped by occupancy)
constexpr int kFlowMaxPerSm = 8;           // bound used to size the progress words
constexpr uint32_t kFlowMinAmps = 64;      // dataflow forward: fewest amplitudes of a chunk per CTA
constexpr int64_t kVjpItemAmps = 65536;    // default amplitudes per VJP work item
constexpr int kTeamCluster = 8;            // CTAs per cluster for the large instances of a ragged batch
constexpr size_t kAlign = 256;

// Smallest single instance that runs on the whole grid (dataflow / cooperative kernels) instead of
// one CTA; MM_GRID_MIN_AMPS overrides it (read once).
int64_t grid_min_amps() {
  static const int64_t v = [] {
    const char* e = getenv("MM_GRID_MIN_AMPS");
    return e ? std::max<int64_t>(64, atoll(e)) : kGridMinAmps;
  }();
  return v;
}


int cuda_fail(cudaError_t e) {
  snprintf(g_last_cuda_error, sizeof(g_last_cuda_error), "%s: %s", cudaGetErrorName(e), cudaGetErrorString(e));
  return MM_ERR_CUDA;
}
#define MM_CUDA(call)                        \
  do {                                       \
    cudaError_t _e = (call);                 \
    if (_e != cudaSuccess) return cuda_fail(_e); \
  } while (0)
#define MM_LAUNCHED()                            \
  do {                                           \
    g_launches.fetch_add(1);                     \
    cudaError_t _e = cudaGetLastError();         \
    if (_e != cudaSuccess) return cuda_fail(_e); \
  } while (0)

uint64_t wait_budget_ns() {
  static uint64_t v = [] {
    const char* s = getenv("MM_WAIT_BUDGET_NS");
    return s ? strtoull(s, nullptr, 10) : 2000000000ull;
  }();
  return v;
}

struct DevInfo {
  int sms = 0;
  int coop = 0;
};

int device_info(DevInfo& di) {
  static std::mutex mu;
  static DevInfo cache[64];
  static bool have[64] = {};
  int dev = 0;
  int ndev = 0;
  cudaError_t e = cudaGetDeviceCount(&ndev);
  if (e != cudaSuccess || ndev == 0) {
    cudaGetLastError();
    return MM_ERR_NO_DEVICE;
  }
  MM_CUDA(cudaGetDevice(&dev));
  std::lock_guard<std::mutex> lk(mu);
  if (dev < 64 && have[dev]) {
    di = cache[dev];
    return MM_OK;
  }
  MM_CUDA(cudaDeviceGetAttribute(&di.sms, cudaDevAttrMultiProcessorCount, dev));
  MM_CUDA(cudaDeviceGetAttribute(&di.coop, cudaDevAttrCooperativeLaunch, dev));
  if (dev < 64) {
    cache[dev] = di;
    have[dev] = true;
  }
  return MM_OK;
}

size_t align_up(size_t x) { return (x + kAlign - 1) / kAlign * kAlign; }

// Fill a Geom from D and a host shape; checks every limit of the kernels.
int make_geom(int D, const int64_t* shape, Geom& g) {
  if (D < 1 || shape == nullptr) return MM_ERR_INVALID_ARG;
  if (D > MM_MAXD) return MM_ERR_UNSUPPORTED;
  memset(&g, 0, sizeof(g));
  g.D = D;
  int64_t n = 1, sumC = 0;
  int32_t maxC = 0;
  for (int i = 0; i < D; ++i) {
    if (shape[i] < 1) return MM_ERR_INVALID_ARG;
    if (shape[i] > (int64_t)INT32_MAX / 2) return MM_ERR_TOO_LARGE;
    if (n > ((int64_t)1 << 62) / shape[i]) return MM_ERR_TOO_LARGE;
    n *= shape[i];
    g.shape[i] = shape[i];
    g.prefC[i] = (int32_t)sumC;
    sumC += shape[i];
    maxC = std::max<int32_t>(maxC, (int32_t)shape[i]);
  }
  if (sumC > (int64_t)INT32_MAX / 2) return MM_ERR_TOO_LARGE;
  g.strides[D - 1] = 1;
  for (int i = D - 1; i > 0; --i) g.strides[i - 1] = g.strides[i] * g.shape[i];
  // chunk / fiber / prefix indices are 32-bit
  if (g.strides[0] > (int64_t)INT32_MAX) return MM_ERR_TOO_LARGE;
  if (n / g.shape[D - 1] > (int64_t)INT32_MAX) return MM_ERR_TOO_LARGE;
  g.n = n;
  g.sumC = sumC;
  g.maxC = maxC;
  return MM_OK;
}

// VJP work split of one instance: fibers per item and item count.
void vjp_split(const Geom& g, int64_t target_amps, uint32_t& fpi, int64_t& items) {
  const int64_t s0 = g.strides[0], C0 = g.shape[0];
  int64_t f = (target_amps + C0 - 1) / C0;
  f = (f + MM_BLOCK - 1) / MM_BLOCK * MM_BLOCK;
  if (f < MM_BLOCK) f = MM_BLOCK;
  if (f > s0) f = s0;
  fpi = (uint32_t)f;
  items = (s0 + f - 1) / f;
}

// Workspace regions shared by every entry point.
struct Layout {
  size_t tables = 0, coef = 0, partials = 0, desc = 0, order = 0, big = 0, items = 0, flags = 0, total = 0;
  int64_t kmax = 0, n_flags = 0;
};

Layout make_layout(int64_t kmax, int64_t coef_entries_total, int64_t n_items, int64_t n_desc, int64_t n_order,
                   int64_t n_flags = 0) {
  Layout L;
  L.kmax = kmax;
  L.n_flags = n_flags;
  size_t off = sizeof(WsHeader);
  L.tables = off;
  off = align_up(off + 3 * (size_t)kmax * sizeof(double));
  L.coef = off;
  off = align_up(off + (size_t)coef_entries_total * sizeof(double2));
  L.partials = off;
  off = align_up(off + (size_t)n_items * MM_NV_MAX * sizeof(double2));
  L.desc = off;
  off = align_up(off + (size_t)n_desc * sizeof(InstDesc));
  L.order = off;
  off = align_up(off + (size_t)n_order * sizeof(int32_t));
  L.big = off;
  off = align_up(off + (size_t)n_order * sizeof(int32_t));
  L.items = off;
  off = align_up(off + (size_t)n_items * sizeof(VjpItem));
  L.flags = off;
  off = align_up(off + (size_t)n_flags * sizeof(uint32_t));
  L.total = off;
  return L;
}

// Uniform (one shape) plan of a call.
struct UniformPlan {
  Geom g;
  int64_t B;
  uint32_t fpi;
  int64_t items_per_inst;
  Layout L;
};

// `fwd`: the plan includes the progress words of the dataflow forward (the last
// workspace region, which the VJP does not use).
int plan_uniform(int64_t B, int D, const int64_t* shape, UniformPlan& P, int sms, bool fwd = true) {
  int rc = make_geom(D, shape, P.g);
  if (rc) return rc;
  if (B < 0) return MM_ERR_INVALID_ARG;
  P.B = B;
  // enough VJP items to fill the GPU several times over
  const int64_t total = B * P.g.n;
  int64_t want_items = std::max<int64_t>((total + kVjpItemAmps - 1) / kVjpItemAmps, 4 * (int64_t)std::max(sms, 1));
  int64_t per_inst = std::max<int64_t>(1, (want_items + std::max<int64_t>(B, 1) - 1) / std::max<int64_t>(B, 1));
  int64_t target = std::max<int64_t>(1, P.g.n / per_inst);
  vjp_split(P.g, target, P.fpi, P.items_per_inst);
  // progress words of the dataflow forward (one large instance)
  const int64_t n_flags =
      (fwd && B == 1 && P.g.n >= grid_min_amps())
          ? 1 + (int64_t)MM_MAXD * kFlowMaxPerSm * std::max(sms, 1) + (int64_t)kFlowMaxSmid
          : 0;
  P.L = make_layout(P.g.maxC + 1, B * coef_entries(P.g), B * P.items_per_inst, 0, 0, n_flags);
  return MM_OK;
}

int check_ws(void* ws, size_t ws_bytes, size_t need) {
  if (ws == nullptr || ((uintptr_t)ws % kAlign) != 0 || ws_bytes < need) return MM_ERR_WORKSPACE;
  return MM_OK;
}

UniformSrc uniform_src(const UniformPlan& P, const double2* A, const double2* b, const double2* c, double2* G,
                       const double2* dLdG, char* ws) {
  UniformSrc s;
  s.g = P.g;
  s.B = P.B;
  s.A = A;
  s.b = b;
  s.c = c;
  s.G = G;
  s.dLdG = dLdG;
  s.coef = reinterpret_cast<double2*>(ws + P.L.coef);
  s.coef_stride = coef_entries(P.g);
  s.items_per_inst = P.items_per_inst;
  s.fibers_per_item = P.fpi;
  return s;
}

Tables tables_of(char* ws, const Layout& L) {
  Tables T;
  double* base = reinterpret_cast<double*>(ws + L.tables);
  T.sq = base;
  T.rs = base + L.kmax;
  T.hh = base + 2 * L.kmax;
  T.kmax = L.kmax;
  return T;
}

int reset_launch_state(char* ws, cudaStream_t st) {
  MM_CUDA(cudaMemsetAsync(ws + MM_WS_LAUNCH_STATE_OFFSET, 0, MM_WS_LAUNCH_STATE_BYTES, st));
  return MM_OK;
}

template <class Src>
int launch_setup(const Src& src, int64_t n_inst, char* ws, const Layout& L, int do_coef, cudaStream_t st) {
  double* base = reinterpret_cast<double*>(ws + L.tables);
  int64_t blocks = std::max<int64_t>(1, std::min<int64_t>(do_coef ? n_inst : 1, 65535));
  blocks = std::max<int64_t>(blocks, std::min<int64_t>((L.kmax + 255) / 256, 65535));
  setup_kernel<Src><<<(unsigned)blocks, 256, 0, st>>>(src, base, base + L.kmax, base + 2 * L.kmax, L.kmax, do_coef);
  MM_LAUNCHED();
  return MM_OK;
}

// Tuning of the dataflow forward; MM_FLOW_BLOCK, MM_FLOW_PER_SM, MM_FLOW_MIN_AMPS
// and MM_FLOW_EXCLUSIVE in the environment override the defaults.
// poll: G is filled with kPendingBits first and every range polls the amplitudes of other CTAs
// that it reads, instead of waiting on their progress words (when every level below the
// shared-memory face runs on lane-pair ranges; MM_FLOW_POLL=0: progress words).
struct FlowTuning {
  int block = kFlowBlock, per_sm = kFlowPerSm, exclusive = 1, poll = 1;
  uint32_t min_amps = kFlowMinAmps;
};

FlowTuning flow_tuning() {
  static FlowTuning t = [] {
    FlowTuning r;
    if (const char* e = getenv("MM_FLOW_BLOCK")) r.block = std::min(256, std::max(32, atoi(e)) / 32 * 32);
    if (const char* e = getenv("MM_FLOW_PER_SM")) r.per_sm = std::min(kFlowMaxPerSm, std::max(1, atoi(e)));
    if (const char* e = getenv("MM_FLOW_MIN_AMPS")) r.min_amps = (uint32_t)std::max(2, atoi(e));
    if (const char* e = getenv("MM_FLOW_EXCLUSIVE")) r.exclusive = atoi(e) != 0;
    if (const char* e = getenv("MM_FLOW_POLL")) r.poll = atoi(e) != 0;
    return r;
  }();
  return t;
}

// One small instance on one thread-block cluster (fwd_cluster_kernel, no setup
// kernel): used for single vanilla instances of at least MM_CLUSTER_MIN_AMPS
// amplitudes (default 1024) that fit its shared-memory tables (cluster_fits);
// MM_CLUSTER_FWD=0 disables it, MM_CLUSTER_CTAS fixes the cluster size (default:
// CTA 0 for slab 0 plus one worker CTA per 64 amplitudes of a level-0 chunk, at
// most 16 CTAs).
struct ClusterTuning {
  int enabled = 1, ctas = 0;
  int64_t min_amps = 1024;
};
ClusterTuning cluster_tuning() {
  static ClusterTuning t = [] {
    ClusterTuning r;
    if (const char* e = getenv("MM_CLUSTER_FWD")) r.enabled = atoi(e) != 0;
    if (const char* e = getenv("MM_CLUSTER_CTAS")) r.ctas = std::min(16, std::max(1, atoi(e)));
    if (const char* e = getenv("MM_CLUSTER_MIN_AMPS")) r.min_amps = std::max<int64_t>(1, atoll(e));
    return r;
  }();
  return t;
}

bool cluster_route(const UniformPlan& P, int stable) {
  const ClusterTuning t = cluster_tuning();
  return P.B == 1 && !stable && t.enabled && P.g.n >= t.min_amps && cluster_fits(P.g);
}

template <int D, int A>
int launch_fwd_cluster_A(const UniformSrc& src, int cl, cudaStream_t st) {
  auto kern = fwd_cluster_kernel<D, A>;
  // attributes once per kernel; whether a cluster of `cl` fits, once per (kernel, cl)
  static std::once_flag attr_once;
  static std::atomic<int> fits[17];
  std::call_once(attr_once, [&] {
    cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)cluster_fwd_smem_bytes());
    cudaFuncSetAttribute(kern, cudaFuncAttributeNonPortableClusterSizeAllowed, 1);
    cudaGetLastError();
  });
  cudaLaunchAttribute attr[1];
  cudaLaunchConfig_t cfg = {};
  attr[0].id = cudaLaunchAttributeClusterDimension;
  attr[0].val.clusterDim.x = (unsigned)cl;
  attr[0].val.clusterDim.y = 1;
  attr[0].val.clusterDim.z = 1;
  cfg.gridDim = dim3((unsigned)cl);
  cfg.blockDim = dim3(256);
  cfg.dynamicSmemBytes = cluster_fwd_smem_bytes();
  cfg.stream = st;
  cfg.attrs = attr;
  cfg.numAttrs = 1;
  int f = fits[cl].load();
  if (f == 0) {
    int ncl = 0;
    f = (cudaOccupancyMaxActiveClusters(&ncl, kern, &cfg) == cudaSuccess && ncl >= 1) ? 1 : -1;
    cudaGetLastError();
    fits[cl].store(f);
  }
  if (f < 0) return MM_ERR_UNSUPPORTED;
  MM_CUDA(cudaLaunchKernelEx(&cfg, kern, src));
  g_launches.fetch_add(1);
  return MM_OK;
}

template <int D>
int launch_fwd_cluster_D(const UniformPlan& P, const UniformSrc& src, cudaStream_t st) {
  const ClusterTuning t = cluster_tuning();
  const uint32_t s0 = (uint32_t)P.g.strides[0];
  int cl = t.ctas ? t.ctas : (s0 <= 64u ? 1 : (int)std::min<uint32_t>(16u, 1u + (s0 + 63u) / 64u));
  int rc = MM_ERR_UNSUPPORTED;
  for (; cl >= 1 && rc == MM_ERR_UNSUPPORTED; cl = cl > 8 ? 8 : 0) {
    const uint32_t nwork = cl > 1 ? (uint32_t)cl - 1u : 1u;
    const uint32_t pc = (s0 + nwork - 1u) / nwork;
    if (pc > kClusterRangeMax) break;
    if (pc <= 128) rc = launch_fwd_cluster_A<D, 1>(src, cl, st);
    else if (pc <= 256) rc = launch_fwd_cluster_A<D, 2>(src, cl, st);
    else rc = launch_fwd_cluster_A<D, 4>(src, cl, st);
  }
  return rc;
}

int launch_fwd_cluster(const UniformPlan& P, const UniformSrc& src, cudaStream_t st) {
  switch (P.g.D) {
    case 1: return launch_fwd_cluster_D<1>(P, src, st);
    case 2: return launch_fwd_cluster_D<2>(P, src, st);
    case 3: return launch_fwd_cluster_D<3>(P, src, st);
    case 4: return launch_fwd_cluster_D<4>(P, src, st);
    case 5: return launch_fwd_cluster_D<5>(P, src, st);
    case 6: return launch_fwd_cluster_D<6>(P, src, st);
    case 7: return launch_fwd_cluster_D<7>(P, src, st);
    case 8: return launch_fwd_cluster_D<8>(P, src, st);
  }
  return MM_ERR_UNSUPPORTED;
}

template <int D>
int launch_fwd_uniform_D(const UniformPlan& P, const UniformSrc& src, char* ws, int stable, const DevInfo& di,
                         cudaStream_t st) {
  const double* rs = tables_of(ws, P.L).rs;
  WsHeader* h = reinterpret_cast<WsHeader*>(ws);
  if (P.B == 1 && P.g.n >= grid_min_amps() && di.coop && stable) {
    int per_sm = 0;
    MM_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, stable_grid_kernel<D>, kGridBlock, 0));
    if (per_sm >= 1) {
      uint64_t budget = wait_budget_ns();
      UniformSrc s = src;
      void* args[] = {&s, (void*)&rs, &h, &budget};
      MM_CUDA(cudaLaunchCooperativeKernel((void*)stable_grid_kernel<D>, dim3(di.sms), dim3(kGridBlock), args, 0, st));
      g_launches.fetch_add(1);
      return MM_OK;
    }
  }
  if (P.B == 1 && P.g.n >= grid_min_amps() && di.coop && !stable) {
    const FlowTuning t = flow_tuning();
    int occ = 0;
    MM_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, fwd_flow_kernel<D>, t.block, 0));
    if (occ >= 1) {
      const int per_sm = std::min(occ, t.per_sm);
      FlowPlan fp;
      const int64_t n_flags = flow_plan(P.g, di.sms, per_sm, t.min_amps, t.exclusive, wait_budget_ns(), fp);
      // progress words, then the SM registration words
      if (n_flags + (int64_t)kFlowMaxSmid > P.L.n_flags) return MM_ERR_WORKSPACE;
      uint32_t* prog = reinterpret_cast<uint32_t*>(ws + P.L.flags);
      bool poll = t.poll;
      for (int i = 0; poll && i < (int)fp.small_lvl && i < D; ++i)
        poll = fp.ctas[i] > 1 && fp.per[i] <= 2u * (uint32_t)t.block;
      if (poll) {  // every amplitude reads as pending until written (G[0] is read from c)
        fp.poll_halo = 1;
        MM_CUDA(cudaMemsetAsync(src.G, 0xff, (size_t)P.g.n * sizeof(double2), st));
      }
      MM_CUDA(cudaMemsetAsync(prog, 0, (size_t)(n_flags + kFlowMaxSmid) * sizeof(uint32_t), st));
      UniformSrc s = src;
      void* args[] = {&s, (void*)&rs, &h, &prog, &fp};
      MM_CUDA(cudaLaunchCooperativeKernel((void*)fwd_flow_kernel<D>, dim3(per_sm * di.sms), dim3(t.block), args, 0,
                                          st));
      g_launches.fetch_add(1);
      return MM_OK;
    }
  }
  if (P.B > 0) {
    fwd_cta_kernel<D, D, UniformSrc><<<(unsigned)P.B, MM_BLOCK, 0, st>>>(src, rs, stable);
    MM_LAUNCHED();
  }
  return MM_OK;
}

int launch_fwd_uniform(const UniformPlan& P, const UniformSrc& src, char* ws, int stable, const DevInfo& di,
                       cudaStream_t st) {
  switch (P.g.D) {
    case 1: return launch_fwd_uniform_D<1>(P, src, ws, stable, di, st);
    case 2: return launch_fwd_uniform_D<2>(P, src, ws, stable, di, st);
    case 3: return launch_fwd_uniform_D<3>(P, src, ws, stable, di, st);
    case 4: return launch_fwd_uniform_D<4>(P, src, ws, stable, di, st);
    case 5: return launch_fwd_uniform_D<5>(P, src, ws, stable, di, st);
    case 6: return launch_fwd_uniform_D<6>(P, src, ws, stable, di, st);
    case 7: return launch_fwd_uniform_D<7>(P, src, ws, stable, di, st);
    case 8: return launch_fwd_uniform_D<8>(P, src, ws, stable, di, st);
  }
  return MM_ERR_UNSUPPORTED;
}

template <class Src>
int launch_vjp_items(int D, const Src& src, Tables T, double2* partials, int64_t item_base, int64_t n_items,
                     cudaStream_t st) {
  if (n_items <= 0) return MM_OK;
  // gridDim.x limit is 2^31 - 1; split very long item lists
  for (int64_t done = 0; done < n_items;) {
    const unsigned nb = (unsigned)std::min<int64_t>(n_items - done, INT32_MAX);
    const int64_t base = item_base + done;
    switch (D) {
      case 1: vjp_items_kernel<1, 1, Src><<<nb, MM_BLOCK, 0, st>>>(src, T, partials, base); break;
      case 2: vjp_items_kernel<2, 2, Src><<<nb, MM_BLOCK, 0, st>>>(src, T, partials, base); break;
      case 3: vjp_items_kernel<3, 3, Src><<<nb, MM_BLOCK, 0, st>>>(src, T, partials, base); break;
      case 4: vjp_items_kernel<4, 4, Src><<<nb, MM_BLOCK, 0, st>>>(src, T, partials, base); break;
      case 5: vjp_items_kernel<5, 5, Src><<<nb, MM_BLOCK, 0, st>>>(src, T, partials, base); break;
      case 6: vjp_items_kernel<6, 6, Src><<<nb, MM_BLOCK, 0, st>>>(src, T, partials, base); break;
      case 7: vjp_items_kernel<7, 7, Src><<<nb, MM_BLOCK, 0, st>>>(src, T, partials, base); break;
      case 8: vjp_items_kernel<8, 8, Src><<<nb, MM_BLOCK, 0, st>>>(src, T, partials, base); break;
      default: return MM_ERR_UNSUPPORTED;
    }
    MM_LAUNCHED();
    done += nb;
  }
  return MM_OK;
}

template <class Src>
int launch_vjp_reduce(const Src& src, int64_t n_inst, const double2* partials, double2* dA, double2* db, double2* dc,
                      cudaStream_t st) {
  if (n_inst <= 0) return MM_OK;
  const int64_t blocks = (n_inst + 3) / 4;
  vjp_reduce_kernel<Src><<<(unsigned)blocks, 128, 0, st>>>(src, partials, dA, db, dc);
  MM_LAUNCHED();
  return MM_OK;
}

int common_checks(void* ws, mm_stream_t stream, DevInfo& di) {
  (void)ws;
  (void)stream;
  return device_info(di);
}

}  // namespace

// ======================================================================= ABI
struct mm_ragged_plan {
  int64_t B = 0;
  std::vector<InstDesc> desc;
  std::vector<int32_t> order;     // forward schedule: instances by decreasing cost
  std::vector<int32_t> small;     // instances run by one CTA each (decreasing cost)
  std::vector<int32_t> big;       // instances run by a cluster each (decreasing cost)
  std::vector<VjpItem> items;     // VJP items grouped by D, then instance
  std::vector<int64_t> d_item_begin, d_item_count;  // per D (index D)
  int maxD = 0;
  int64_t kmax = 0;
  int64_t total_amps = 0;
  int64_t total_coef = 0;
  int64_t team_min_amps = 0;
  int team_cluster = kTeamCluster;  // CTAs per cluster team (1 = no teams)
  int64_t vjp_item_amps = kVjpItemAmps;
  int copy_split = 0;  // eighths of the instances whose host copy of G the forward writes
  Layout L;
};

namespace {
int ragged_build(mm_ragged_plan* p) {
  const int64_t B = p->B;
  // large instances (at least team_min_amps amplitudes) go to cluster teams
  int64_t thr = p->team_min_amps;
  if (thr == 0) thr = std::max<int64_t>(65536, p->total_amps / (4 * 152));  // about 1/4 of an SM's share
  p->small.clear();
  p->big.clear();
  for (int32_t k : p->order)
    (p->team_cluster > 1 && p->desc[k].g.n >= thr ? p->big : p->small).push_back(k);
  // VJP items: one launch over every item; instances by decreasing cost, so the
  // largest items are scheduled first (longest-processing-time order)
  p->items.clear();
  p->d_item_begin.assign(MM_MAXD + 1, 0);
  p->d_item_count.assign(MM_MAXD + 1, 0);
  for (int32_t k : p->order) {
    InstDesc& d = p->desc[k];
    uint32_t fpi;
    int64_t nit;
    vjp_split(d.g, p->vjp_item_amps, fpi, nit);
    d.item_begin = (int64_t)p->items.size();
    d.n_items = nit;
    d.fibers_per_item = fpi;
    p->d_item_count[d.g.D] += nit;
    for (int64_t r = 0; r < nit; ++r) {
      VjpItem it;
      it.inst = k;
      it.q0 = (uint32_t)(r * fpi);
      it.q1 = (uint32_t)std::min<int64_t>((r + 1) * (int64_t)fpi, d.g.strides[0]);
      it.pad = 0;
      p->items.push_back(it);
    }
  }
  (void)B;
  p->L = make_layout(p->kmax, p->total_coef, (int64_t)p->items.size(), p->B, p->B);
  return MM_OK;
}

RaggedSrc ragged_src(const mm_ragged_plan* p, char* ws, const double2* A, const double2* b, const double2* c,
                     double2* G, const double2* dLdG) {
  RaggedSrc s;
  s.desc = reinterpret_cast<const InstDesc*>(ws + p->L.desc);
  s.order = reinterpret_cast<const int32_t*>(ws + p->L.order);
  s.B = p->B;
  s.A = A;
  s.b = b;
  s.c = c;
  s.G = G;
  s.dLdG = dLdG;
  s.coef = reinterpret_cast<double2*>(ws + p->L.coef);
  s.items = reinterpret_cast<const VjpItem*>(ws + p->L.items);
  s.Gout = nullptr;
  s.fwd_copy_eighths = p->copy_split;
  return s;
}
}  // namespace

namespace {
template <int DHI>
int launch_team_D(const mm_ragged_plan* p, const RaggedSrc& src, char* w, const double* rs, int stable,
                  cudaStream_t st) {
  auto kern = fwd_ragged_team_kernel<1, DHI>;
  const int cl = p->team_cluster;
  if (cl > 8) MM_CUDA(cudaFuncSetAttribute(kern, cudaFuncAttributeNonPortableClusterSizeAllowed, 1));
  cudaLaunchConfig_t cfg = {};
  cudaLaunchAttribute attr[1];
  attr[0].id = cudaLaunchAttributeClusterDimension;
  attr[0].val.clusterDim.x = cl;
  attr[0].val.clusterDim.y = 1;
  attr[0].val.clusterDim.z = 1;
  cfg.blockDim = dim3(MM_BLOCK);
  cfg.dynamicSmemBytes = 0;
  cfg.stream = st;
  cfg.attrs = attr;
  cfg.numAttrs = 1;
  cfg.gridDim = dim3(cl);
  int ncl = 0;
  MM_CUDA(cudaOccupancyMaxActiveClusters(&ncl, kern, &cfg));
  if (ncl < 1) return MM_ERR_UNSUPPORTED;
  cfg.gridDim = dim3((unsigned)(ncl * cl));
  const int32_t* small = reinterpret_cast<const int32_t*>(w + p->L.big);
  const int32_t* big = small + p->small.size();
  WsHeader* h = reinterpret_cast<WsHeader*>(w);
  MM_CUDA(cudaLaunchKernelEx(&cfg, kern, src, rs, stable, big, (int)p->big.size(), small, (int)p->small.size(), h));
  g_launches.fetch_add(1);
  return MM_OK;
}

int launch_ragged_team(const mm_ragged_plan* p, const RaggedSrc& src, char* w, const double* rs, int stable,
                       cudaStream_t st) {
  if (p->maxD <= 2) return launch_team_D<2>(p, src, w, rs, stable, st);
  if (p->maxD <= 4) return launch_team_D<4>(p, src, w, rs, stable, st);
  return launch_team_D<8>(p, src, w, rs, stable, st);
}
}  // namespace

void mm::note_launches(int64_t n) { g_launches.fetch_add(n); }

// ------------------------------------------------------- host-buffer entry points
// Per device: one pinned staging area and one device buffer (workspace, inputs, outputs), grown
// on demand and reused; a call holds the device's mutex from the first copy to the last.
namespace {
struct HostStage {
  std::mutex mu;
  char* pin = nullptr;
  size_t pin_bytes = 0;
  char* dev = nullptr;
  size_t dev_bytes = 0;
  bool ws_fresh = false;
  size_t ws_at = 0;  // offset of the workspace in `dev` at the last call
};
HostStage g_stage[64];

int stage_reserve(HostStage& s, size_t pin_need, size_t dev_need) {
  if (s.pin_bytes < pin_need) {
    if (s.pin) MM_CUDA(cudaFreeHost(s.pin));
    s.pin = nullptr;
    s.pin_bytes = 0;
    MM_CUDA(cudaMallocHost(reinterpret_cast<void**>(&s.pin), pin_need));
    s.pin_bytes = pin_need;
  }
  if (s.dev_bytes < dev_need) {
    if (s.dev) MM_CUDA(cudaFree(s.dev));
    s.dev = nullptr;
    s.dev_bytes = 0;
    MM_CUDA(cudaMalloc(reinterpret_cast<void**>(&s.dev), dev_need));
    s.dev_bytes = dev_need;
    s.ws_fresh = true;
  }
  return MM_OK;
}

// Runs `compute` on `ins` (host buffers, concatenated into the pinned staging area) and copies
// `outs` back.  Device buffer: outputs, then the workspace (its status word right after the
// outputs, so one copy brings both back), then device copies of the inputs.  With `zero_copy_in`
// the kernels read the inputs from the pinned staging area itself (mapped into the device's
// address space), which saves the upload for small inputs read once.
struct HostSeg {
  const void* host;
  size_t bytes;
};
struct HostOut {
  void* host;
  size_t bytes;
};
template <class F>
int run_host_staged(size_t ws_bytes, const HostSeg* ins, int n_in, const HostOut* outs, int n_out, cudaStream_t st,
                    bool zero_copy_in, F compute) {
  int dev = 0;
  MM_CUDA(cudaGetDevice(&dev));
  HostStage& s = g_stage[dev & 63];
  std::lock_guard<std::mutex> lk(s.mu);
  size_t in_bytes = 0, out_bytes = 0;
  for (int i = 0; i < n_in; ++i) in_bytes += align_up(ins[i].bytes);
  for (int i = 0; i < n_out; ++i) out_bytes += align_up(outs[i].bytes);
  const size_t d_ws = out_bytes, d_in = d_ws + align_up(ws_bytes);
  const size_t p_out = in_bytes;  // pinned: inputs, then outputs and the status word
  int rc = stage_reserve(s, p_out + out_bytes + kAlign, d_in + (zero_copy_in ? 0 : in_bytes));
  if (rc) return rc;
  char* ws = s.dev + d_ws;
  if (s.ws_fresh || s.ws_at != d_ws) {  // the workspace moved (or is new): zero its header
    MM_CUDA(cudaMemsetAsync(ws, 0, sizeof(WsHeader), st));
    s.ws_fresh = false;
    s.ws_at = d_ws;
  }
  std::vector<char*> din(n_in), dout(n_out);
  size_t o = 0;
  for (int i = 0; i < n_in; ++i) {
    memcpy(s.pin + o, ins[i].host, ins[i].bytes);
    din[i] = zero_copy_in ? s.pin + o : s.dev + d_in + o;
    o += align_up(ins[i].bytes);
  }
  if (in_bytes && !zero_copy_in) MM_CUDA(cudaMemcpyAsync(s.dev + d_in, s.pin, in_bytes, cudaMemcpyHostToDevice, st));
  o = 0;
  for (int i = 0; i < n_out; ++i) {
    dout[i] = s.dev + o;
    o += align_up(outs[i].bytes);
  }
  if ((rc = compute(ws, din.data(), dout.data()))) return rc;
  // outputs and the status word (first bytes of the workspace, right after them) in one copy
  MM_CUDA(cudaMemcpyAsync(s.pin + p_out, s.dev, out_bytes + sizeof(int32_t), cudaMemcpyDeviceToHost, st));
  MM_CUDA(cudaStreamSynchronize(st));
  int32_t status = 0;
  memcpy(&status, s.pin + p_out + out_bytes, sizeof(status));
  if (status != 0) {
    MM_CUDA(cudaMemsetAsync(ws, 0, sizeof(int32_t), st));
    MM_CUDA(cudaStreamSynchronize(st));
    return status;
  }
  o = 0;
  for (int i = 0; i < n_out; ++i) {
    memcpy(outs[i].host, s.pin + p_out + o, outs[i].bytes);
    o += align_up(outs[i].bytes);
  }
  return MM_OK;
}
}  // namespace

// Host-buffer forward of one instance on the one-cluster kernel: the kernel reads A, b, c from
// the pinned staging area and writes G straight into it (the GPU addresses pinned host memory
// directly; the kernel never reads G back), so the call is one launch, one synchronisation and
// one host copy.  The kernel has no waits that can give up, so there is no status word to read.
namespace {
int fwd_host_cluster(const UniformPlan& P, const mm_c128* A, const mm_c128* b, const mm_c128* c, mm_c128* G,
                     cudaStream_t st) {
  int dev = 0;
  MM_CUDA(cudaGetDevice(&dev));
  HostStage& s = g_stage[dev & 63];
  std::lock_guard<std::mutex> lk(s.mu);
  const int D = P.g.D;
  const size_t a_bytes = align_up((size_t)D * D * sizeof(mm_c128)), b_bytes = align_up((size_t)D * sizeof(mm_c128));
  const size_t in_bytes = a_bytes + b_bytes + align_up(sizeof(mm_c128));
  const size_t out_bytes = (size_t)P.g.n * sizeof(mm_c128);
  int rc = stage_reserve(s, in_bytes + out_bytes, 0);
  if (rc) return rc;
  memcpy(s.pin, A, (size_t)D * D * sizeof(mm_c128));
  memcpy(s.pin + a_bytes, b, (size_t)D * sizeof(mm_c128));
  memcpy(s.pin + a_bytes + b_bytes, c, sizeof(mm_c128));
  UniformSrc src = uniform_src(P, reinterpret_cast<const double2*>(s.pin), reinterpret_cast<const double2*>(s.pin + a_bytes),
                               reinterpret_cast<const double2*>(s.pin + a_bytes + b_bytes),
                               reinterpret_cast<double2*>(s.pin + in_bytes), nullptr, s.pin);
  src.coef = nullptr;  // no workspace: the cluster kernel builds its own coefficients
  if ((rc = launch_fwd_cluster(P, src, st))) return rc;
  MM_CUDA(cudaStreamSynchronize(st));
  memcpy(G, s.pin + in_bytes, out_bytes);
  return MM_OK;
}
}  // namespace

// Binomial fill: the forward's workspace (setup tables), then the fill state,
// the composition-count table and the per-CTA wave sums.  The waves run in up
// to three launches picked from their sizes n_w (known on the host): waves of
// at most MM_BLOCK amplitudes on one CTA, waves of at most one amplitude per
// thread of a cluster on one thread-block cluster, larger waves on a
// cooperative grid; each launch continues from the fill state the previous one
// left (and returns at once when that state says the fill has stopped).
namespace {
constexpr int64_t kBnMaxW1 = 1 << 24;
constexpr int kBnMaxTeam = 16;
constexpr int kBnMaxPerSm = 2;
// Staged operands per CTA: every CTA copies them at launch, so a large prefix
// permutation (108 KB at 30^4) costs more to stage than its L2 reads (measured).
// With the kernel's static shared memory this stays under the 48 KB a launch may
// use without opting in.
constexpr size_t kBnStageBytes = 40 * 1024;
constexpr int64_t kBnMaxPerm = 1 << 24;  // prefixes beyond this: no permutation (binary-search unranking)

struct BinomialPlan {
  int64_t W1 = 0;      // max weight + 1
  int64_t W1p = 0;     // max weight of the prefix axes 0 .. D-2, + 1
  int64_t P = 0;       // prefixes (flat index over the axes 0 .. D-2); 0: no prefix permutation
  int64_t last = 0;    // last wave the reference would fill: global cutoff - 1, capped at the max weight
  int64_t w_team = 0;  // first wave of the cluster launch
  int64_t w_grid = 0;  // first wave of the grid launch
  size_t off_state = 0, off_table = 0, off_sp = 0, off_perm = 0, off_part = 0, total = 0;
};

int binomial_env(const char* name, int dflt) {
  const char* e = getenv(name);
  return e ? atoi(e) : dflt;
}

// Workspace layout (team / grid only bound the wave-sum buffer).
int binomial_layout(const UniformPlan& P, int sms, BinomialPlan& B) {
  int64_t wmax = 0;
  for (int i = 0; i < P.g.D; ++i) wmax += P.g.shape[i] - 1;
  B.W1 = wmax + 1;
  if (B.W1 > kBnMaxW1) return MM_ERR_TOO_LARGE;
  B.W1p = B.W1 - (P.g.shape[P.g.D - 1] - 1);
  B.P = P.g.n / P.g.shape[P.g.D - 1];
  if (B.P > kBnMaxPerm) B.P = 0;  // the waves then unrank their indices by binary search
  const int parts = std::max(kBnMaxTeam, kBnMaxPerSm * sms);
  B.off_state = align_up(P.L.total);
  B.off_table = B.off_state + align_up(sizeof(BinomialState));
  B.off_sp = B.off_table + align_up((size_t)(P.g.D + 1) * (size_t)B.W1 * sizeof(int64_t));
  B.off_perm = B.off_sp + (B.P ? align_up((size_t)P.g.D * (size_t)B.W1p * sizeof(int64_t)) : 0);
  B.off_part = B.off_perm + (B.P ? align_up((size_t)B.P * sizeof(uint32_t)) : 0);
  B.total = B.off_part + align_up((size_t)2 * parts * sizeof(double));
  return MM_OK;
}

// Wave sizes n_w = number of indices inside the cutoffs with |k| = w.
std::vector<int64_t> binomial_wave_sizes(const Geom& g, int64_t W1) {
  std::vector<int64_t> cnt((size_t)W1, 0), nxt((size_t)W1, 0);
  cnt[0] = 1;
  for (int j = g.D - 1; j >= 0; --j) {
    int64_t run = 0;
    for (int64_t x = 0; x < W1; ++x) {
      run += cnt[(size_t)x];
      if (x >= g.shape[j]) run -= cnt[(size_t)(x - g.shape[j])];
      nxt[(size_t)x] = run;
    }
    cnt.swap(nxt);
  }
  return cnt;
}

cudaLaunchConfig_t cluster_config(cudaLaunchAttribute* attr, int cl, cudaStream_t st) {
  cudaLaunchConfig_t cfg = {};
  attr[0].id = cudaLaunchAttributeClusterDimension;
  attr[0].val.clusterDim.x = (unsigned)cl;
  attr[0].val.clusterDim.y = 1;
  attr[0].val.clusterDim.z = 1;
  cfg.gridDim = dim3((unsigned)cl);
  cfg.blockDim = dim3(MM_BLOCK);
  cfg.dynamicSmemBytes = 0;
  cfg.stream = st;
  cfg.attrs = attr;
  cfg.numAttrs = 1;
  return cfg;
}

// Largest cluster (16, 8, 4, 2 CTAs) of which one can be resident, 0 if none.
template <int D>
int binomial_team_ctas() {
  static std::atomic<int> cached{-1};
  int v = cached.load();
  if (v >= 0) return v;
  auto kern = binomial_wave_kernel<D, 1>;
  int best = 0;
  if (cudaFuncSetAttribute(kern, cudaFuncAttributeNonPortableClusterSizeAllowed, 1) == cudaSuccess) {
    for (int cl : {16, 8, 4, 2}) {
      cudaLaunchAttribute attr[1];
      cudaLaunchConfig_t cfg = cluster_config(attr, cl, nullptr);
      cfg.dynamicSmemBytes = kBnStageBytes;  // the most a launch stages
      int ncl = 0;
      if (cudaOccupancyMaxActiveClusters(&ncl, kern, &cfg) == cudaSuccess && ncl >= 1) {
        best = cl;
        break;
      }
    }
  }
  cudaGetLastError();
  cached.store(best);
  return best;
}

// No early stop: the vanilla forward over the whole tensor (every amplitude of
// weight <= last is the binomial fill's), then the mask above `last` and the
// norm of what is kept.
int launch_binomial_nostop(const UniformPlan& P, const BinomialPlan& B, const UniformSrc& src, char* w,
                           double* norm_out, const DevInfo& di, cudaStream_t st) {
  int rc;
  if ((rc = launch_fwd_uniform(P, src, w, 0, di, st))) return rc;
  double* part = reinterpret_cast<double*>(w + B.off_part);
  const int blocks = (int)std::min<int64_t>((P.g.n + 255) / 256, (int64_t)4 * di.sms);
  double2* G = src.G;
  switch (P.g.D) {
#define MM_BN_CASE(DD)                                                                                    \
  case DD:                                                                                                \
    binomial_mask_norm_kernel<DD><<<(unsigned)blocks, 256, 0, st>>>(G, P.g, B.last, part);              \
    break;
    MM_BN_CASE(1)
    MM_BN_CASE(2)
    MM_BN_CASE(3)
    MM_BN_CASE(4)
    MM_BN_CASE(5)
    MM_BN_CASE(6)
    MM_BN_CASE(7)
    MM_BN_CASE(8)
#undef MM_BN_CASE
    default:
      return MM_ERR_UNSUPPORTED;
  }
  MM_LAUNCHED();
  binomial_norm_final_kernel<<<1, 32, 0, st>>>(part, blocks, norm_out);
  MM_LAUNCHED();
  return MM_OK;
}

template <int D>
int launch_binomial_D(const UniformPlan& P, const BinomialPlan& B, const UniformSrc& src, char* w, double max_l2,
                      double* norm_out, const DevInfo& di, cudaStream_t st) {
  const double* rs = tables_of(w, P.L).rs;
  const int64_t* S = reinterpret_cast<const int64_t*>(w + B.off_table);
  BinomialState* state = reinterpret_cast<BinomialState*>(w + B.off_state);
  double* part = reinterpret_cast<double*>(w + B.off_part);
  WsHeader* h = reinterpret_cast<WsHeader*>(w);
  const int32_t W1 = (int32_t)B.W1, W1p = (int32_t)B.W1p;
  int64_t* Sp = B.P ? reinterpret_cast<int64_t*>(w + B.off_sp) : nullptr;
  uint32_t* perm = B.P ? reinterpret_cast<uint32_t*>(w + B.off_perm) : nullptr;
  if (!binomial_env("MM_BINOMIAL_PERM", 1)) perm = nullptr;
  uint64_t budget = wait_budget_ns();
  // stage the read-only operands in shared memory as far as they fit kBnStageBytes,
  // the most frequently read first
  BinomialStage stage = {};
  const int32_t table_n = (int32_t)((P.g.D + 1) * B.W1);
  const int32_t sp_n = perm ? (int32_t)(P.g.D * B.W1p) : 0;
  const int32_t coef_n = (int32_t)std::min<int64_t>(coef_entries(P.g), INT32_MAX);
  const int32_t rs_n = P.g.maxC + 1;
  const int32_t perm_n = perm ? (int32_t)B.P : 0;
  if (binomial_env("MM_BINOMIAL_STAGE", 1)) {
    auto fits = [&](const BinomialStage& t) { return bn_stage_bytes(t) <= kBnStageBytes; };
    BinomialStage t = stage;
    t.table_n = table_n;
    t.sp_n = sp_n;
    if (fits(t)) stage = t;
    t = stage;
    t.coef_n = coef_n;
    t.rs_n = rs_n;
    if (fits(t)) stage = t;
    t = stage;
    t.perm_n = perm_n;
    if (fits(t)) stage = t;
  }
  const size_t smem = bn_stage_bytes(stage);  // <= kBnStageBytes: no opt-in attribute needed
  binomial_table_kernel<<<perm ? 2 : 1, 256, 0, st>>>(P.g, W1, const_cast<int64_t*>(S), W1p, Sp);
  MM_LAUNCHED();
  if (perm) {
    const unsigned pb = (unsigned)std::min<int64_t>((B.P + 255) / 256, (int64_t)4 * di.sms);
    binomial_perm_kernel<<<pb, 256, 0, st>>>(P.g, Sp, W1p, perm, B.P);
    MM_LAUNCHED();
  }

  // launch split
  int team = binomial_env("MM_BINOMIAL_TEAM", -1);
  team = team < 0 ? binomial_team_ctas<D>() : std::min(team, binomial_team_ctas<D>());
  int grid = 0;
  if (di.coop && binomial_env("MM_BINOMIAL_GRID", 1)) {
    int occ = 0;
    MM_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, binomial_wave_kernel<D, 2>, MM_BLOCK, smem));
    const int per_sm = std::min({occ, kBnMaxPerSm, std::max(1, binomial_env("MM_BINOMIAL_GRID_PER_SM", 1))});
    grid = per_sm >= 1 ? per_sm * di.sms : 0;
  }
  const std::vector<int64_t> n = binomial_wave_sizes(P.g, B.W1);
  const int64_t last = B.last;
  // threads of the one-CTA and cluster launches (64, 128 or 256)
  int nt = binomial_env("MM_BINOMIAL_BLOCK", MM_BLOCK);
  nt = nt <= 64 ? 64 : nt <= 128 ? 128 : MM_BLOCK;
  const int64_t cta_items = std::max(1, binomial_env("MM_BINOMIAL_CTA_ITEMS", nt));
  const int64_t team_items = std::max<int64_t>(cta_items, binomial_env("MM_BINOMIAL_TEAM_ITEMS", team * nt));
  int64_t w_team = 1;
  while (w_team <= last && n[(size_t)w_team] <= cta_items) ++w_team;
  int64_t w_grid = w_team;
  if (team > 0)
    while (w_grid <= last && n[(size_t)w_grid] <= team_items) ++w_grid;
  if (grid <= 0) w_grid = last + 1;               // no cooperative grid: the cluster (or the CTA) goes on
  if (team <= 0 && grid <= 0) w_team = last + 1;  // neither: one CTA fills every wave
  if (team <= 0) w_team = w_grid;

  binomial_wave_kernel<D, 0><<<1, nt, smem, st>>>(src, rs, S, W1, Sp, W1p, perm, stage, 1, (int32_t)w_team,
                                                        max_l2, part, state, norm_out, h, budget);
  MM_LAUNCHED();
  if (w_team < w_grid) {
    auto kern = binomial_wave_kernel<D, 1>;
    cudaLaunchAttribute attr[1];
    cudaLaunchConfig_t cfg = cluster_config(attr, team, st);
    cfg.blockDim = dim3((unsigned)nt);
    cfg.dynamicSmemBytes = smem;
    const int32_t wb = (int32_t)w_team, we = (int32_t)w_grid;
    const int64_t* Spc = Sp;
    const uint32_t* permc = perm;
    MM_CUDA(cudaLaunchKernelEx(&cfg, kern, src, rs, S, W1, Spc, W1p, permc, stage, wb, we, max_l2, part, state,
                               norm_out, h, budget));
    g_launches.fetch_add(1);
  }
  if (w_grid <= last) {
    UniformSrc s = src;
    int32_t wb = (int32_t)w_grid, we = (int32_t)(last + 1);
    const int64_t* Spc = Sp;
    const uint32_t* permc = perm;
    void* args[] = {&s,      (void*)&rs, (void*)&S, (void*)&W1, (void*)&Spc, (void*)&W1p, (void*)&permc, &stage,
                    &wb,     &we,        &max_l2,   &part,      &state,      &norm_out,   &h,            &budget};
    MM_CUDA(cudaLaunchCooperativeKernel((void*)binomial_wave_kernel<D, 2>, dim3((unsigned)grid), dim3(MM_BLOCK), args,
                                        smem, st));
    g_launches.fetch_add(1);
  }
  return MM_OK;
}
}  // namespace

extern "C" {

const char* mm_status_string(int status) {
  switch (status) {
    case MM_OK: return "ok";
    case MM_ERR_INVALID_ARG: return "invalid argument";
    case MM_ERR_UNSUPPORTED: return "unsupported number of modes";
    case MM_ERR_TOO_LARGE: return "tensor too large for the kernels' 32-bit slab indices";
    case MM_ERR_CUDA: return "CUDA runtime error";
    case MM_ERR_WAIT_TIMEOUT: return "bounded inter-CTA wait timed out";
    case MM_ERR_WORKSPACE: return "workspace missing, misaligned or too small";
    case MM_ERR_NO_DEVICE: return "no CUDA device";
  }
  return "unknown status";
}

int mm_max_modes(void) { return MM_MAXD; }
const char* mm_last_cuda_error(void) { return g_last_cuda_error; }
int64_t mm_launch_count(void) { return g_launches.load(); }

int mm_workspace_init(void* ws, size_t ws_bytes, mm_stream_t stream) {
  if (ws == nullptr || ws_bytes < sizeof(WsHeader)) return MM_ERR_WORKSPACE;
  MM_CUDA(cudaMemsetAsync(ws, 0, sizeof(WsHeader), (cudaStream_t)stream));
  return MM_OK;
}

int mm_workspace_status(void* ws, mm_stream_t stream, int* status) {
  if (ws == nullptr || status == nullptr) return MM_ERR_INVALID_ARG;
  MM_CUDA(cudaStreamSynchronize((cudaStream_t)stream));
  int32_t v = 0;
  MM_CUDA(cudaMemcpy(&v, ws, sizeof(v), cudaMemcpyDeviceToHost));
  MM_CUDA(cudaMemset(ws, 0, sizeof(int32_t)));
  *status = v;
  return MM_OK;
}

size_t mm_hermite_workspace_bytes(int D, const int64_t* shape, int64_t batch) {
  DevInfo di;
  int sms = device_info(di) == MM_OK ? di.sms : 152;
  UniformPlan P;
  if (plan_uniform(batch < 1 ? 1 : batch, D, shape, P, sms)) return 0;
  return P.L.total;
}

int mm_hermite_fwd_batched(int64_t B, int D, const int64_t* shape, const mm_c128* A, const mm_c128* b,
                           const mm_c128* c, int stable, mm_c128* G, void* ws, size_t ws_bytes, mm_stream_t stream) {
  DevInfo di;
  int rc = common_checks(ws, stream, di);
  if (rc) return rc;
  UniformPlan P;
  if ((rc = plan_uniform(B, D, shape, P, di.sms))) return rc;
  if (B == 0) return MM_OK;
  if (!A || !b || !c || !G) return MM_ERR_INVALID_ARG;
  if ((rc = check_ws(ws, ws_bytes, P.L.total))) return rc;
  cudaStream_t st = (cudaStream_t)stream;
  char* w = static_cast<char*>(ws);
  UniformSrc src = uniform_src(P, (const double2*)A, (const double2*)b, (const double2*)c, (double2*)G, nullptr, w);
  if (cluster_route(P, stable)) {  // one launch, no setup kernel and no workspace state
    rc = launch_fwd_cluster(P, src, st);
    if (rc != MM_ERR_UNSUPPORTED) return rc;  // no cluster fits: the paths below
  }
  if ((rc = reset_launch_state(w, st))) return rc;
  if ((rc = launch_setup(src, B, w, P.L, 1, st))) return rc;
  return launch_fwd_uniform(P, src, w, stable, di, st);
}

int mm_hermite_fwd(int D, const int64_t* shape, const mm_c128* A, const mm_c128* b, const mm_c128* c, int stable,
                   mm_c128* G, void* ws, size_t ws_bytes, mm_stream_t stream) {
  return mm_hermite_fwd_batched(1, D, shape, A, b, c, stable, G, ws, ws_bytes, stream);
}

int mm_hermite_fwd_host(int D, const int64_t* shape, const mm_c128* A, const mm_c128* b, const mm_c128* c, int stable,
                        mm_c128* G, mm_stream_t stream) {
  DevInfo di;
  int rc = device_info(di);
  if (rc) return rc;
  UniformPlan P;
  if ((rc = plan_uniform(1, D, shape, P, di.sms))) return rc;
  if (!A || !b || !c || !G) return MM_ERR_INVALID_ARG;
  if (cluster_route(P, stable)) {
    rc = fwd_host_cluster(P, A, b, c, G, (cudaStream_t)stream);
    if (rc != MM_ERR_UNSUPPORTED) return rc;  // no cluster fits: the staged path below
  }
  const size_t wsb = mm_hermite_workspace_bytes(D, shape, 1);
  const HostSeg ins[3] = {{A, (size_t)D * D * sizeof(mm_c128)}, {b, (size_t)D * sizeof(mm_c128)}, {c, sizeof(mm_c128)}};
  const HostOut outs[1] = {{G, (size_t)P.g.n * sizeof(mm_c128)}};
  return run_host_staged(wsb, ins, 3, outs, 1, (cudaStream_t)stream, true, [&](char* ws, char** din, char** dout) {
    return mm_hermite_fwd(D, shape, (const mm_c128*)din[0], (const mm_c128*)din[1], (const mm_c128*)din[2], stable,
                          (mm_c128*)dout[0], ws, wsb, stream);
  });
}

int mm_hermite_vjp_host(int D, const int64_t* shape, const mm_c128* G, const mm_c128* c, const mm_c128* dLdG,
                        mm_c128* dA, mm_c128* db, mm_c128* dc, mm_stream_t stream) {
  DevInfo di;
  int rc = device_info(di);
  if (rc) return rc;
  UniformPlan P;
  if ((rc = plan_uniform(1, D, shape, P, di.sms, false))) return rc;
  if (!G || !c || !dLdG || !dA || !db || !dc) return MM_ERR_INVALID_ARG;
  const size_t wsb = mm_hermite_workspace_bytes(D, shape, 1);
  const size_t nb = (size_t)P.g.n * sizeof(mm_c128);
  const HostSeg ins[3] = {{G, nb}, {dLdG, nb}, {c, sizeof(mm_c128)}};
  const HostOut outs[3] = {{dA, (size_t)D * D * sizeof(mm_c128)}, {db, (size_t)D * sizeof(mm_c128)},
                           {dc, sizeof(mm_c128)}};
  return run_host_staged(wsb, ins, 3, outs, 3, (cudaStream_t)stream, false, [&](char* ws, char** din, char** dout) {
    return mm_hermite_vjp(D, shape, (const mm_c128*)din[0], (const mm_c128*)din[2], (const mm_c128*)din[1],
                          (mm_c128*)dout[0], (mm_c128*)dout[1], (mm_c128*)dout[2], ws, wsb, stream);
  });
}

size_t mm_binomial_workspace_bytes(int D, const int64_t* shape) {
  DevInfo di;
  int sms = device_info(di) == MM_OK ? di.sms : 152;
  UniformPlan P;
  if (plan_uniform(1, D, shape, P, sms)) return 0;
  BinomialPlan B;
  if (binomial_layout(P, sms, B)) return 0;
  return B.total;
}

int mm_binomial(int D, const int64_t* shape, const mm_c128* A, const mm_c128* b, const mm_c128* c, double max_l2,
                int64_t global_cutoff, mm_c128* G, double* norm_out, void* ws, size_t ws_bytes, mm_stream_t stream) {
  DevInfo di;
  int rc = common_checks(ws, stream, di);
  if (rc) return rc;
  UniformPlan P;
  if ((rc = plan_uniform(1, D, shape, P, di.sms))) return rc;
  if (!A || !b || !c || !G) return MM_ERR_INVALID_ARG;
  BinomialPlan B;
  if ((rc = binomial_layout(P, di.sms, B))) return rc;
  if ((rc = check_ws(ws, ws_bytes, B.total))) return rc;
  if (P.g.n > (int64_t)INT32_MAX * 256) return MM_ERR_TOO_LARGE;
  int64_t wmax = B.W1 - 1;
  B.last = std::max<int64_t>(0, std::min<int64_t>(global_cutoff - 1, wmax));
  cudaStream_t st = (cudaStream_t)stream;
  char* w = static_cast<char*>(ws);
  UniformSrc src = uniform_src(P, (const double2*)A, (const double2*)b, (const double2*)c, (double2*)G, nullptr, w);
  if ((rc = reset_launch_state(w, st))) return rc;
  if ((rc = launch_setup(src, 1, w, P.L, 1, st))) return rc;
  if (!(max_l2 < HUGE_VAL)) return launch_binomial_nostop(P, B, src, w, norm_out, di, st);
  // amplitudes above the stop wave are never written: zero the whole tensor first
  MM_CUDA(cudaMemsetAsync(G, 0, (size_t)P.g.n * sizeof(double2), st));
  switch (D) {
    case 1: return launch_binomial_D<1>(P, B, src, w, max_l2, norm_out, di, st);
    case 2: return launch_binomial_D<2>(P, B, src, w, max_l2, norm_out, di, st);
    case 3: return launch_binomial_D<3>(P, B, src, w, max_l2, norm_out, di, st);
    case 4: return launch_binomial_D<4>(P, B, src, w, max_l2, norm_out, di, st);
    case 5: return launch_binomial_D<5>(P, B, src, w, max_l2, norm_out, di, st);
    case 6: return launch_binomial_D<6>(P, B, src, w, max_l2, norm_out, di, st);
    case 7: return launch_binomial_D<7>(P, B, src, w, max_l2, norm_out, di, st);
    case 8: return launch_binomial_D<8>(P, B, src, w, max_l2, norm_out, di, st);
  }
  return MM_ERR_UNSUPPORTED;
}

int mm_hermite_vjp_batched(int64_t B, int D, const int64_t* shape, const mm_c128* G, const mm_c128* c,
                           const mm_c128* dLdG, mm_c128* dA, mm_c128* db, mm_c128* dc, void* ws, size_t ws_bytes,
                           mm_stream_t stream) {
  DevInfo di;
  int rc = common_checks(ws, stream, di);
  if (rc) return rc;
  UniformPlan P;
  if ((rc = plan_uniform(B, D, shape, P, di.sms, false))) return rc;
  if (B == 0) return MM_OK;
  if (!G || !c || !dLdG || !dA || !db || !dc) return MM_ERR_INVALID_ARG;
  if ((rc = check_ws(ws, ws_bytes, P.L.total))) return rc;
  cudaStream_t st = (cudaStream_t)stream;
  char* w = static_cast<char*>(ws);
  UniformSrc src =
      uniform_src(P, nullptr, nullptr, (const double2*)c, (double2*)G, (const double2*)dLdG, w);
  if ((rc = reset_launch_state(w, st))) return rc;
  if ((rc = launch_setup(src, B, w, P.L, 0, st))) return rc;
  double2* partials = reinterpret_cast<double2*>(w + P.L.partials);
  if ((rc = launch_vjp_items(D, src, tables_of(w, P.L), partials, 0, B * P.items_per_inst, st))) return rc;
  return launch_vjp_reduce(src, B, partials, (double2*)dA, (double2*)db, (double2*)dc, st);
}

int mm_hermite_vjp(int D, const int64_t* shape, const mm_c128* G, const mm_c128* c, const mm_c128* dLdG, mm_c128* dA,
                   mm_c128* db, mm_c128* dc, void* ws, size_t ws_bytes, mm_stream_t stream) {
  return mm_hermite_vjp_batched(1, D, shape, G, c, dLdG, dA, db, dc, ws, ws_bytes, stream);
}

// ------------------------------------------------------------------- ragged
int mm_ragged_plan_create(int64_t B, const int32_t* D, const int64_t* shapes, mm_ragged_plan** plan) {
  if (plan == nullptr || B < 0 || (B > 0 && (D == nullptr || shapes == nullptr))) return MM_ERR_INVALID_ARG;
  if (B > INT32_MAX) return MM_ERR_TOO_LARGE;
  mm_ragged_plan* p = new (std::nothrow) mm_ragged_plan();
  if (!p) return MM_ERR_INVALID_ARG;
  p->B = B;
  p->desc.resize(B);
  int64_t off_g = 0, off_a = 0, off_b = 0, off_coef = 0, off_s = 0;
  for (int64_t k = 0; k < B; ++k) {
    InstDesc& d = p->desc[k];
    memset(&d, 0, sizeof(d));
    int rc = make_geom(D[k], shapes + off_s, d.g);
    if (rc) {
      delete p;
      return rc;
    }
    off_s += D[k];
    d.g_off = off_g;
    d.a_off = off_a;
    d.b_off = off_b;
    d.coef_off = off_coef;
    off_g += d.g.n;
    off_a += (int64_t)D[k] * D[k];
    off_b += D[k];
    off_coef += coef_entries(d.g);
    p->maxD = std::max(p->maxD, (int)D[k]);
    p->kmax = std::max<int64_t>(p->kmax, d.g.maxC + 1);
  }
  p->total_amps = off_g;
  p->total_coef = off_coef;
  p->order.resize(B);
  for (int64_t k = 0; k < B; ++k) p->order[k] = (int32_t)k;
  // largest first: cost ~ amplitudes * (D + 1) terms
  std::stable_sort(p->order.begin(), p->order.end(), [&](int32_t a, int32_t b) {
    return p->desc[a].g.n * (p->desc[a].g.D + 1) > p->desc[b].g.n * (p->desc[b].g.D + 1);
  });
  ragged_build(p);
  *plan = p;
  return MM_OK;
}

void mm_ragged_plan_destroy(mm_ragged_plan* plan) { delete plan; }
size_t mm_ragged_plan_workspace_bytes(const mm_ragged_plan* plan) { return plan ? plan->L.total : 0; }
int64_t mm_ragged_plan_amplitudes(const mm_ragged_plan* plan) { return plan ? plan->total_amps : 0; }

int mm_ragged_plan_offsets(const mm_ragged_plan* plan, int64_t* g_off, int64_t* a_off, int64_t* b_off) {
  if (!plan) return MM_ERR_INVALID_ARG;
  for (int64_t k = 0; k < plan->B; ++k) {
    if (g_off) g_off[k] = plan->desc[k].g_off;
    if (a_off) a_off[k] = plan->desc[k].a_off;
    if (b_off) b_off[k] = plan->desc[k].b_off;
  }
  return MM_OK;
}

int mm_ragged_plan_set_tuning(mm_ragged_plan* plan, int64_t team_min_amps, int64_t vjp_item_amps) {
  if (!plan || team_min_amps < 0 || vjp_item_amps < 1) return MM_ERR_INVALID_ARG;
  plan->team_min_amps = team_min_amps;
  plan->vjp_item_amps = vjp_item_amps;
  return ragged_build(plan);
}

int mm_ragged_plan_set_copy_split(mm_ragged_plan* plan, int eighths) {
  if (!plan || eighths < 0 || eighths > 8) return MM_ERR_INVALID_ARG;
  plan->copy_split = eighths;
  return MM_OK;
}

int mm_ragged_plan_set_team_size(mm_ragged_plan* plan, int cluster_ctas) {
  if (!plan || (cluster_ctas != 1 && cluster_ctas != 2 && cluster_ctas != 4 && cluster_ctas != 8 &&
                cluster_ctas != 16))
    return MM_ERR_INVALID_ARG;
  plan->team_cluster = cluster_ctas;
  return ragged_build(plan);
}

int mm_ragged_plan_upload(const mm_ragged_plan* plan, void* ws, size_t ws_bytes, mm_stream_t stream) {
  if (!plan) return MM_ERR_INVALID_ARG;
  DevInfo di;
  int rc = device_info(di);
  if (rc) return rc;
  if ((rc = check_ws(ws, ws_bytes, plan->L.total))) return rc;
  cudaStream_t st = (cudaStream_t)stream;
  char* w = static_cast<char*>(ws);
  if (plan->B > 0) {
    MM_CUDA(cudaMemcpyAsync(w + plan->L.desc, plan->desc.data(), plan->desc.size() * sizeof(InstDesc),
                            cudaMemcpyHostToDevice, st));
    MM_CUDA(cudaMemcpyAsync(w + plan->L.order, plan->order.data(), plan->order.size() * sizeof(int32_t),
                            cudaMemcpyHostToDevice, st));
    std::vector<int32_t> lists(plan->small);
    lists.insert(lists.end(), plan->big.begin(), plan->big.end());
    MM_CUDA(cudaMemcpyAsync(w + plan->L.big, lists.data(), lists.size() * sizeof(int32_t), cudaMemcpyHostToDevice,
                            st));
  }
  if (!plan->items.empty())
    MM_CUDA(cudaMemcpyAsync(w + plan->L.items, plan->items.data(), plan->items.size() * sizeof(VjpItem),
                            cudaMemcpyHostToDevice, st));
  MM_CUDA(cudaStreamSynchronize(st));
  return MM_OK;
}

int mm_ragged_fwd(const mm_ragged_plan* plan, const mm_c128* A, const mm_c128* b, const mm_c128* c, int stable,
                  mm_c128* G, void* ws, size_t ws_bytes, mm_stream_t stream) {
  return mm_ragged_fwd_copy_g(plan, A, b, c, stable, G, nullptr, ws, ws_bytes, stream);
}

int mm_ragged_fwd_copy_g(const mm_ragged_plan* plan, const mm_c128* A, const mm_c128* b, const mm_c128* c,
                         int stable, mm_c128* G, mm_c128* G_copy, void* ws, size_t ws_bytes, mm_stream_t stream) {
  if (!plan) return MM_ERR_INVALID_ARG;
  DevInfo di;
  int rc = device_info(di);
  if (rc) return rc;
  if (plan->B == 0) return MM_OK;
  if (!A || !b || !c || !G) return MM_ERR_INVALID_ARG;
  if ((rc = check_ws(ws, ws_bytes, plan->L.total))) return rc;
  cudaStream_t st = (cudaStream_t)stream;
  char* w = static_cast<char*>(ws);
  RaggedSrc src = ragged_src(plan, w, (const double2*)A, (const double2*)b, (const double2*)c, (double2*)G, nullptr);
  src.Gout = (double2*)G_copy;  // the instances of the forward's share (copy_split) also go there
  if ((rc = reset_launch_state(w, st))) return rc;
  if ((rc = launch_setup(src, plan->B, w, plan->L, 1, st))) return rc;
  const double* rs = tables_of(w, plan->L).rs;
  if (!plan->big.empty()) return launch_ragged_team(plan, src, w, rs, stable, st);
  const unsigned nb = (unsigned)plan->B;
  if (plan->maxD <= 2) fwd_cta_kernel<1, 2, RaggedSrc><<<nb, MM_BLOCK, 0, st>>>(src, rs, stable);
  else if (plan->maxD <= 4) fwd_cta_kernel<1, 4, RaggedSrc><<<nb, MM_BLOCK, 0, st>>>(src, rs, stable);
  else fwd_cta_kernel<1, 8, RaggedSrc><<<nb, MM_BLOCK, 0, st>>>(src, rs, stable);
  MM_LAUNCHED();
  return MM_OK;
}

int mm_ragged_vjp(const mm_ragged_plan* plan, const mm_c128* G, const mm_c128* c, const mm_c128* dLdG, mm_c128* dA,
                  mm_c128* db, mm_c128* dc, void* ws, size_t ws_bytes, mm_stream_t stream) {
  return mm_ragged_vjp_copy_g(plan, G, c, dLdG, dA, db, dc, nullptr, ws, ws_bytes, stream);
}

int mm_ragged_vjp_copy_g(const mm_ragged_plan* plan, const mm_c128* G, const mm_c128* c, const mm_c128* dLdG,
                         mm_c128* dA, mm_c128* db, mm_c128* dc, mm_c128* G_copy, void* ws, size_t ws_bytes,
                         mm_stream_t stream) {
  if (!plan) return MM_ERR_INVALID_ARG;
  DevInfo di;
  int rc = device_info(di);
  if (rc) return rc;
  if (plan->B == 0) return MM_OK;
  if (!G || !c || !dLdG || !dA || !db || !dc) return MM_ERR_INVALID_ARG;
  if ((rc = check_ws(ws, ws_bytes, plan->L.total))) return rc;
  cudaStream_t st = (cudaStream_t)stream;
  char* w = static_cast<char*>(ws);
  RaggedSrc src = ragged_src(plan, w, nullptr, nullptr, (const double2*)c, (double2*)G, (const double2*)dLdG);
  src.Gout = (double2*)G_copy;
  if ((rc = reset_launch_state(w, st))) return rc;
  if ((rc = launch_setup(src, plan->B, w, plan->L, 0, st))) return rc;
  double2* partials = reinterpret_cast<double2*>(w + plan->L.partials);
  Tables T = tables_of(w, plan->L);
  const int64_t n_items = (int64_t)plan->items.size();
  for (int64_t done = 0; done < n_items;) {
    const unsigned nb = (unsigned)std::min<int64_t>(n_items - done, INT32_MAX);
    if (G_copy == nullptr) {
      if (plan->maxD <= 2) vjp_items_kernel<1, 2, RaggedSrc><<<nb, MM_BLOCK, 0, st>>>(src, T, partials, done);
      else if (plan->maxD <= 4) vjp_items_kernel<1, 4, RaggedSrc><<<nb, MM_BLOCK, 0, st>>>(src, T, partials, done);
      else vjp_items_kernel<1, 8, RaggedSrc><<<nb, MM_BLOCK, 0, st>>>(src, T, partials, done);
    } else {
      if (plan->maxD <= 2) vjp_items_kernel<1, 2, RaggedSrc, true><<<nb, MM_BLOCK, 0, st>>>(src, T, partials, done);
      else if (plan->maxD <= 4)
        vjp_items_kernel<1, 4, RaggedSrc, true><<<nb, MM_BLOCK, 0, st>>>(src, T, partials, done);
      else vjp_items_kernel<1, 8, RaggedSrc, true><<<nb, MM_BLOCK, 0, st>>>(src, T, partials, done);
    }
    MM_LAUNCHED();
    done += nb;
  }
  return launch_vjp_reduce(src, plan->B, partials, (double2*)dA, (double2*)db, (double2*)dc, st);
}

// ------------------------------------------------------------ checkpointed VJP
}  // extern "C"
namespace {
// Segments of kseg slabs along axis 0; checkpoint buffer = slab 0, then the two
// slabs before each later segment (s - 2, s - 1 for s = j * kseg).
struct CkptPlan {
  UniformPlan P;
  int kseg = 0;
  int64_t nseg = 0;
  size_t win = 0, total = 0;
};

int plan_ckpt(int D, const int64_t* shape, int kseg, int sms, CkptPlan& cp) {
  if (kseg < 2) return MM_ERR_INVALID_ARG;
  int rc = plan_uniform(1, D, shape, cp.P, sms, false);
  if (rc) return rc;
  const Geom& g = cp.P.g;
  cp.kseg = kseg;
  cp.nseg = (g.shape[0] + kseg - 1) / kseg;
  cp.P.L = make_layout(g.maxC + 1, coef_entries(g), cp.nseg * cp.P.items_per_inst, 0, 0, 0);
  cp.win = cp.P.L.total;
  const int64_t slabs = std::min<int64_t>(kseg, g.shape[0]) + 2;
  cp.total = align_up(cp.win + (size_t)slabs * (size_t)g.strides[0] * sizeof(double2));
  return MM_OK;
}

int64_t ckpt_slabs(int64_t C0, int kseg) { return 1 + 2 * (((C0 + kseg - 1) / kseg) - 1); }

template <int D>
int launch_ckpt_segments(const CkptPlan& cp, const UniformSrc& src, char* w, const double2* ckpt, double2* dA,
                         double2* db, double2* dc, cudaStream_t st) {
  const Geom& g = cp.P.g;
  const int64_t s0 = g.strides[0], C0 = g.shape[0];
  double2* W = reinterpret_cast<double2*>(w + cp.win);
  const Tables T = tables_of(w, cp.P.L);
  double2* partials = reinterpret_cast<double2*>(w + cp.P.L.partials);
  const int64_t items = cp.P.items_per_inst;
  UniformSrc ws = src;
  ws.G = W;
  const unsigned nb = (unsigned)((s0 + 255) / 256);
  for (int64_t j = 0; j < cp.nseg; ++j) {
    const int s = (int)(j * cp.kseg), e = (int)std::min<int64_t>(s + cp.kseg, C0);
    const int wbase = j == 0 ? 0 : s - 2;
    const double2* from = j == 0 ? ckpt : ckpt + s0 + 2 * (j - 1) * s0;
    MM_CUDA(cudaMemcpyAsync(W, from, (size_t)(j == 0 ? 1 : 2) * s0 * sizeof(double2), cudaMemcpyDeviceToDevice, st));
    for (int m = j == 0 ? 1 : s; m < e; ++m) {
      fwd_slab_kernel<D><<<nb, 256, 0, st>>>(g, src.b, src.coef, T.rs, W, m, wbase);
      MM_LAUNCHED();
    }
    vjp_window_kernel<D><<<(unsigned)items, MM_BLOCK, 0, st>>>(ws, T, partials + j * items * MM_NV_MAX, s, e, wbase);
    MM_LAUNCHED();
  }
  UniformSrc rs = src;
  rs.items_per_inst = cp.nseg * items;
  return launch_vjp_reduce(rs, 1, partials, dA, db, dc, st);
}
}  // namespace
extern "C" {

int64_t mm_hermite_checkpoint_elems(int D, const int64_t* shape, int kseg) {
  Geom g;
  if (kseg < 2 || make_geom(D, shape, g)) return -1;
  return ckpt_slabs(g.shape[0], kseg) * g.strides[0];
}

int mm_hermite_checkpoint_save(int D, const int64_t* shape, int kseg, const mm_c128* G, mm_c128* ckpt,
                               mm_stream_t stream) {
  Geom g;
  int rc = make_geom(D, shape, g);
  if (rc) return rc;
  if (kseg < 2 || !G || !ckpt) return MM_ERR_INVALID_ARG;
  cudaStream_t st = (cudaStream_t)stream;
  const int64_t s0 = g.strides[0], nseg = (g.shape[0] + kseg - 1) / kseg;
  const size_t slab = (size_t)s0 * sizeof(mm_c128);
  MM_CUDA(cudaMemcpyAsync(ckpt, G, slab, cudaMemcpyDeviceToDevice, st));
  for (int64_t j = 1; j < nseg; ++j)
    MM_CUDA(cudaMemcpyAsync(ckpt + s0 + 2 * (j - 1) * s0, G + (j * kseg - 2) * s0, 2 * slab, cudaMemcpyDeviceToDevice,
                            st));
  return MM_OK;
}

size_t mm_hermite_vjp_checkpointed_workspace_bytes(int D, const int64_t* shape, int kseg) {
  DevInfo di;
  int sms = device_info(di) == MM_OK ? di.sms : 152;
  CkptPlan cp;
  if (plan_ckpt(D, shape, kseg, sms, cp)) return 0;
  return cp.total;
}

int mm_hermite_vjp_checkpointed(int D, const int64_t* shape, int kseg, const mm_c128* A, const mm_c128* b,
                                const mm_c128* c, const mm_c128* ckpt, const mm_c128* dLdG, mm_c128* dA, mm_c128* db,
                                mm_c128* dc, void* ws, size_t ws_bytes, mm_stream_t stream) {
  DevInfo di;
  int rc = device_info(di);
  if (rc) return rc;
  CkptPlan cp;
  if ((rc = plan_ckpt(D, shape, kseg, di.sms, cp))) return rc;
  if (!A || !b || !c || !ckpt || !dLdG || !dA || !db || !dc) return MM_ERR_INVALID_ARG;
  if ((rc = check_ws(ws, ws_bytes, cp.total))) return rc;
  cudaStream_t st = (cudaStream_t)stream;
  char* w = static_cast<char*>(ws);
  UniformSrc src = uniform_src(cp.P, (const double2*)A, (const double2*)b, (const double2*)c, nullptr,
                               (const double2*)dLdG, w);
  if ((rc = reset_launch_state(w, st))) return rc;
  if ((rc = launch_setup(src, 1, w, cp.P.L, 1, st))) return rc;
  double2 *oA = (double2*)dA, *ob = (double2*)db, *oc = (double2*)dc;
  const double2* ck = (const double2*)ckpt;
  int r2 = MM_ERR_UNSUPPORTED;
  switch (D) {
    case 1: r2 = launch_ckpt_segments<1>(cp, src, w, ck, oA, ob, oc, st); break;
    case 2: r2 = launch_ckpt_segments<2>(cp, src, w, ck, oA, ob, oc, st); break;
    case 3: r2 = launch_ckpt_segments<3>(cp, src, w, ck, oA, ob, oc, st); break;
    case 4: r2 = launch_ckpt_segments<4>(cp, src, w, ck, oA, ob, oc, st); break;
    case 5: r2 = launch_ckpt_segments<5>(cp, src, w, ck, oA, ob, oc, st); break;
    case 6: r2 = launch_ckpt_segments<6>(cp, src, w, ck, oA, ob, oc, st); break;
    case 7: r2 = launch_ckpt_segments<7>(cp, src, w, ck, oA, ob, oc, st); break;
    case 8: r2 = launch_ckpt_segments<8>(cp, src, w, ck, oA, ob, oc, st); break;
  }
  return r2;
}

// ------------------------------------------------------- VJP without a workspace
// Scratch of mm_hermite_vjp_noalloc: MM_NOALLOC_SCRATCH_BYTES (2 MiB, include/mm_gb300.h)
// of device memory in this library's module, present on every GPU that loads the
// library until the process exits.
static __device__ __align__(256) unsigned char g_vjp_scratch[MM_NOALLOC_SCRATCH_BYTES];

// Device address of g_vjp_scratch for the current device, looked up once per
// device (cudaGetSymbolAddress, with that device current) and cached.
static int noalloc_scratch(void** out) {
  static std::mutex mu;
  static void* addr[64] = {};
  int dev = 0;
  MM_CUDA(cudaGetDevice(&dev));
  if (dev < 0 || dev >= 64) return MM_ERR_UNSUPPORTED;
  std::lock_guard<std::mutex> lk(mu);
  if (addr[dev] == nullptr) {
    void* p = nullptr;
    MM_CUDA(cudaGetSymbolAddress(&p, g_vjp_scratch));
    addr[dev] = p;
  }
  *out = addr[dev];
  return MM_OK;
}

int mm_hermite_vjp_noalloc(int D, const int64_t* shape, const mm_c128* G, const mm_c128* c, const mm_c128* dLdG,
                           mm_c128* dA, mm_c128* db, mm_c128* dc, mm_stream_t stream) {
  DevInfo di;
  int rc = device_info(di);
  if (rc) return rc;
  UniformPlan P;
  if ((rc = plan_uniform(1, D, shape, P, di.sms, false))) return rc;
  if (P.L.total > MM_NOALLOC_SCRATCH_BYTES) return MM_ERR_TOO_LARGE;
  // every argument is checked before the shared array is touched: a rejected call has no
  // effect on the device (it cannot disturb a call still running on another stream)
  if (!G || !c || !dLdG || !dA || !db || !dc) return MM_ERR_INVALID_ARG;
  void* ws = nullptr;
  if ((rc = noalloc_scratch(&ws))) return rc;
  // the status word is the only scratch content read before it is written
  MM_CUDA(cudaMemsetAsync(ws, 0, sizeof(WsHeader), (cudaStream_t)stream));
  return mm_hermite_vjp(D, shape, G, c, dLdG, dA, db, dc, ws, MM_NOALLOC_SCRATCH_BYTES, stream);
}

// ---------------------------------------------------------------- diagnostics
int mm_selftest(void* ws, size_t ws_bytes, mm_stream_t stream, int* nbad) {
  DevInfo di;
  int rc = device_info(di);
  if (rc) return rc;
  if (!nbad) return MM_ERR_INVALID_ARG;
  if ((rc = check_ws(ws, ws_bytes, 8192))) return rc;
  cudaStream_t st = (cudaStream_t)stream;
  char* w = static_cast<char*>(ws);
  const int64_t shape[3] = {12, 10, 11};
  UniformPlan P;
  if ((rc = plan_uniform(2, 3, shape, P, di.sms))) return rc;
  // real addresses inside the workspace; only c is ever read by the kernel
  double2* A = reinterpret_cast<double2*>(w + 512);
  double2* b = reinterpret_cast<double2*>(w + 1024);
  double2* c = reinterpret_cast<double2*>(w + 1280);
  double2* G = reinterpret_cast<double2*>(w + 1536);
  double2* dLdG = reinterpret_cast<double2*>(w + 1792);
  double2* coef = reinterpret_cast<double2*>(w + 2048);
  InstDesc* desc = reinterpret_cast<InstDesc*>(w + 4096);
  InstView* expect = reinterpret_cast<InstView*>(w + 4608);
  int32_t* bad = reinterpret_cast<int32_t*>(w + 5120);
  int32_t* order = reinterpret_cast<int32_t*>(w + 5632);
  const double2 cv[2] = {make_double2(0.25, -0.5), make_double2(-1.5, 2.75)};
  MM_CUDA(cudaMemcpyAsync(c, cv, sizeof(cv), cudaMemcpyHostToDevice, st));
  int total_bad = 0;
  for (int pass = 0; pass < 2; ++pass) {
    InstView e;
    memset(&e, 0, sizeof(e));
    const int64_t k = pass == 0 ? 1 : 0;
    if (pass == 0) {
      UniformSrc src = uniform_src(P, A, b, c, G, dLdG, w);
      src.coef = coef;
      e.g = P.g;
      e.A = A + 9;
      e.b = b + 3;
      e.c = cv[1];
      e.G = G + P.g.n;
      e.dLdG = dLdG + P.g.n;
      e.coef = coef + coef_entries(P.g);
      MM_CUDA(cudaMemcpyAsync(expect, &e, sizeof(e), cudaMemcpyHostToDevice, st));
      view_selftest_kernel<UniformSrc><<<1, 32, 0, st>>>(src, k, expect, bad);
    } else {
      InstDesc d;
      memset(&d, 0, sizeof(d));
      const int64_t shape2[4] = {3, 1, 4, 2};
      if ((rc = make_geom(4, shape2, d.g))) return rc;
      d.g_off = 5;
      d.a_off = 7;
      d.b_off = 2;
      d.coef_off = 11;
      MM_CUDA(cudaMemcpyAsync(desc, &d, sizeof(d), cudaMemcpyHostToDevice, st));
      RaggedSrc src;
      memset(&src, 0, sizeof(src));
      src.desc = desc;
      src.order = order;
      src.B = 1;
      src.A = A;
      src.b = b;
      src.c = c;
      src.G = G;
      src.dLdG = dLdG;
      src.coef = coef;
      e.g = d.g;
      e.A = A + 7;
      e.b = b + 2;
      e.c = cv[0];
      e.G = G + 5;
      e.dLdG = dLdG + 5;
      e.coef = coef + 11;
      MM_CUDA(cudaMemcpyAsync(expect, &e, sizeof(e), cudaMemcpyHostToDevice, st));
      view_selftest_kernel<RaggedSrc><<<1, 32, 0, st>>>(src, k, expect, bad);
    }
    MM_LAUNCHED();
    int32_t hb = -1;
    MM_CUDA(cudaMemcpyAsync(&hb, bad, sizeof(hb), cudaMemcpyDeviceToHost, st));
    MM_CUDA(cudaStreamSynchronize(st));
    total_bad += hb;
  }
  *nbad = total_bad;
  return MM_OK;
}

int mm_test_wait_timeout(void* ws, size_t ws_bytes, uint64_t budget_ns, mm_stream_t stream) {
  DevInfo di;
  int rc = device_info(di);
  if (rc) return rc;
  if ((rc = check_ws(ws, ws_bytes, sizeof(WsHeader)))) return rc;
  if (!di.coop) return MM_ERR_UNSUPPORTED;
  cudaStream_t st = (cudaStream_t)stream;
  char* w = static_cast<char*>(ws);
  if ((rc = reset_launch_state(w, st))) return rc;
  WsHeader* h = reinterpret_cast<WsHeader*>(w);
  void* args[] = {&h, &budget_ns};
  MM_CUDA(cudaLaunchCooperativeKernel((void*)wait_timeout_test_kernel, dim3(2), dim3(32), args, 0, st));
  g_launches.fetch_add(1);
  return MM_OK;
}

#ifdef MM_DEVICE_CHECKS
// Debug builds only: this runtime's view of a device pointer, and a copy-engine read of it.
MM_API int mm_debug_ptr_attr(const void* p, int* type, int* device) {
  cudaPointerAttributes a;
  cudaError_t e = cudaPointerGetAttributes(&a, p);
  if (e != cudaSuccess) {
    cuda_fail(e);
    cudaGetLastError();
    return MM_ERR_CUDA;
  }
  *type = (int)a.type;
  *device = a.device;
  return MM_OK;
}
MM_API int mm_debug_read_bytes(const void* dev, void* host, size_t n) {
  MM_CUDA(cudaMemcpy(host, dev, n, cudaMemcpyDeviceToHost));
  return MM_OK;
}
// Debug builds only: copy the first recorded access violation (8 words) to host memory.
MM_API int mm_debug_read(unsigned long long* out8) {
  MM_CUDA(cudaMemcpyFromSymbol(out8, mm::mm_dbg_word, 8 * sizeof(unsigned long long)));
  return MM_OK;
}
#endif

}  // extern "C"
