// engine.cu -- host side of the device engine and the C ABI declared in include/phx.h.
//
// A context owns one device, one stream and one device-memory arena.  An
// instance is one FEM volume: its pattern and scatter map are built on the
// host once (pattern.cpp) and uploaded; all solver state then lives on the
// device.  A solve (or a batch of solves, or a serving loop) runs "rounds" of
// persistent kernels over the packed tile index of the active instances; the
// per-instance state machine (newton_control.h) advances between kernels on
// the device, and the host only reads the active count after each round.
#include <cuda_runtime.h>

#include <algorithm>
#include <atomic>
#include <condition_variable>
#include <memory>
#include <mutex>
#include <new>
#include <system_error>
#include <thread>
#include <chrono>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <deque>
#include <map>
#include <string>
#include <type_traits>
#include <vector>

#include "../../include/phx.h"
#include "errors.h"
#include "kernels.h"
#include "newton_control.h"
#include "pattern.h"
#include "serve_admission.h"

using namespace phx;

namespace {

thread_local std::string g_err;

int set_err(int code, const std::string& msg) {
  g_err = msg;
  return code;
}

}  // namespace

int phx::set_last_error(int code, const std::string& msg) { return set_err(code, msg); }

namespace {

#define CU(call)                                                                              \
  do {                                                                                        \
    cudaError_t e_ = (call);                                                                  \
    if (e_ != cudaSuccess)                                                                    \
      return set_err(PHX_ECUDA, std::string(#call) + ": " + cudaGetErrorString(e_));          \
  } while (0)

using clk = std::chrono::steady_clock;

// wall-clock limit of one blocking solve call (the device never waits; this bounds the host loop)
constexpr double kSolveTimeLimit = 600.0;
// Newton rounds per engine launch in a blocking solve (the host checks completion between launches)
constexpr int kRoundsPerLaunch = 16;

// ---------------------------------------------------------------------------
// device arena: one allocation, first-fit free list with coalescing, 256 B alignment
// ---------------------------------------------------------------------------
struct Arena {
  char* base = nullptr;
  size_t cap = 0, used = 0;
  std::map<size_t, size_t> free_;
  std::map<size_t, size_t> live_;

  cudaError_t init(size_t bytes) {
    cap = (bytes + 255) & ~(size_t)255;
    cudaError_t e = cudaMalloc(&base, cap);
    if (e != cudaSuccess) { base = nullptr; cap = 0; return e; }
    free_[0] = cap;
    return cudaSuccess;
  }
  void release() {
    if (base) cudaFree(base);
    base = nullptr;
    free_.clear();
    live_.clear();
    cap = used = 0;
  }
  void* alloc(size_t bytes) {
    bytes = std::max<size_t>(256, (bytes + 255) & ~(size_t)255);
    for (auto it = free_.begin(); it != free_.end(); ++it) {
      if (it->second >= bytes) {
        size_t off = it->first, sz = it->second;
        free_.erase(it);
        if (sz > bytes) free_[off + bytes] = sz - bytes;
        live_[off] = bytes;
        used += bytes;
        return base + off;
      }
    }
    return nullptr;
  }
  size_t size_of(const void* p) const {
    if (!p) return 0;
    auto it = live_.find((size_t)((const char*)p - base));
    return it == live_.end() ? 0 : it->second;
  }
  void free(void* p) {
    if (!p) return;
    size_t off = (char*)p - base;
    auto it = live_.find(off);
    if (it == live_.end()) return;
    size_t sz = it->second;
    live_.erase(it);
    used -= sz;
    auto nx = free_.lower_bound(off);
    if (nx != free_.end() && off + sz == nx->first) {
      sz += nx->second;
      nx = free_.erase(nx);
    }
    if (nx != free_.begin()) {
      auto pv = std::prev(nx);
      if (pv->first + pv->second == off) {
        pv->second += sz;
        return;
      }
    }
    free_[off] = sz;
  }
};

}  // namespace

struct phx_context_s {
  int device = 0;
  int num_sms = 0;
  cudaStream_t stream = nullptr;
  Arena arena;
  int64_t launches = 0;
  // profiling
  bool profiling = false;
  struct Ev { int kind; cudaEvent_t a, b; };
  std::vector<Ev> evs;
  std::vector<cudaEvent_t> pool;
  double prof_ms[K_COUNT] = {0};
  int64_t prof_n[K_COUNT] = {0};
  // batch buffers
  int cap = 0;
  InstDev* d_inst = nullptr;
  int32_t* d_pre = nullptr;   // 3 * (cap + 1) + 1 (num)
  int32_t* d_flags = nullptr; // 8 + cap
  int32_t* h_flags = nullptr; // pinned mirror
  std::vector<int32_t> h_pre;
  const void* batch_owner = nullptr;  // who set the batch buffers last
  double* d_algo = nullptr;           // [K_COUNT] algorithmic bytes per kernel kind (profiling)
  cudaEvent_t marks[16] = {};
  // engine
  GridBar* d_bar = nullptr;
  int32_t* d_phc = nullptr;  // [32] per-phase instance counts of the engine (live, snapshot)
  int32_t* d_act = nullptr;
  int act_cap = 0;
  unsigned long long* d_stage = nullptr;  // [32] stage ns + executions (profiling)
  int egrid[2] = {0, 0};
  // cluster PCG: the batch's cluster instances (largest first) and the waiting lists the
  // engine writes for the cluster kernels
  int32_t* d_corder = nullptr;  // [cap]
  int32_t* d_wait = nullptr;    // [wait_size(cap)]
  int32_t* d_cfg = nullptr;     // [4]: [0] unused, [1] graph loop passes,
                                // [2] whole-GPU PCG iterations run by the graph
  int ccount = 0;               // instances of the batch whose PCG runs outside the engine
  int ckind_count[4] = {0, 0, 0, 0};  // ... of each PCG kind (1, 2: clusters, 3: whole-GPU kernels)
  int gmax[3] = {-1, -1, -1};   // clusters of kinds 1, 2 resident at once (-1: not queried yet)
  int ggrid = 0;                // CTAs of the whole-GPU PCG kernels
  // scheduling of batch solves (defaults, and tuned settings per batch mix)
  phx_launch_settings launch{1, kWaitRounds, kWaitShare, kRoundsPerLaunch, 0, kSliceShare, kSliceMin};
  std::map<std::string, phx_launch_settings> tuned;
  // pinned landing area of batch downloads (states and positions of a batch, one synchronisation)
  char* down = nullptr;
  size_t down_cap = 0;
  // pinned staging of instance set-ups (grown as needed, reused once its last copy is done)
  char* stage = nullptr;
  size_t stage_cap = 0;
  cudaEvent_t stage_ev = nullptr;
  // the whole solve loop as one graph, kept while the batch and launch parameters stay the same
  cudaGraph_t graph = nullptr;
  cudaGraphExec_t gexec = nullptr;
  std::string gkey;
  long long wait_limit = kBarrierLimit;  // grid-barrier wait limit of the engine (SM cycles)
  int unmet_tag = 0;                     // test hook: grid barrier that waits for an arrival never made
};

// A server's own copy of a cold request's mesh: the instance is built from it at admission
// and rebuilt from it after an eviction.
struct KeptMesh {
  int32_t n = 0, m = 0;
  std::vector<double> X0, lame, rho, force, soft_k, soft_target;
  std::vector<int32_t> T;
  std::vector<uint8_t> model, fixed;
  double gravity[3] = {0, 0, 0};
  phx_mesh view() const {
    phx_mesh v{};
    v.num_nodes = n;
    v.num_tets = m;
    v.X0 = X0.data();
    v.tets = T.data();
    v.lame = lame.data();
    v.rho = rho.data();
    v.model = model.empty() ? nullptr : model.data();
    v.fixed = fixed.empty() ? nullptr : fixed.data();
    v.force = force.empty() ? nullptr : force.data();
    for (int c = 0; c < 3; ++c) v.gravity[c] = gravity[c];
    v.soft_k = soft_k.empty() ? nullptr : soft_k.data();
    v.soft_target = soft_target.empty() ? nullptr : soft_target.data();
    return v;
  }
};

// Host part of a server instance: not built, being built on a worker, ready, or failed.
enum HostState : int { HOST_NONE = 0, HOST_BUILDING = 1, HOST_READY = 2, HOST_FAILED = 3 };

struct phx_instance_s {
  phx_context ctx = nullptr;
  HostPattern hp;
  InstDev dev{};
  std::vector<void*> blocks;
  NState* d_st = nullptr;
  DevOpts* d_opts = nullptr;
  bool have32 = false, have64 = false;
  int64_t bytes = 0;
  bool in_server = false;
  double gravity[3] = {0, 0, 0};
  std::vector<double> force;
  // instances a server created for cold requests (phx_server_submit_mesh): its budget holds
  // their device memory while they are resident, idle ones included
  phx_server owner = nullptr;
  std::unique_ptr<KeptMesh> kept;
  bool resident = true;                    // the device part exists
  std::atomic<int> host_state{HOST_READY};
  std::string host_err;
  std::vector<double> saved_x, saved_v;    // positions and velocities kept on the host by an eviction
  uint64_t last_used = 0;                  // server tick of the last request (eviction order)
  // staged boundary conditions (phx_instance_set_staging): the stage persists across solves
  bool grid_eligible = false;              // FP32 above the cluster size: PCG kind 3 when the launch settings allow
  int32_t stage = 0, num_stages = 0;
  bool stage_values = false;               // a stage moves targets or changes a soft stiffness
  std::vector<double> soft0;               // soft records at stage 0, restored by phx_instance_reset
  std::vector<int32_t> stage_grp;          // host copies of the staging arrays (uploaded again when a
  std::vector<double> stage_ini, stage_par;  // server re-creates the instance after an eviction)
};

// Drops a server-created instance from its server's bookkeeping (defined with the server).
void server_forget(phx_server s, phx_instance inst);
// Adds device bytes of one of its instances to a server's count.
void server_account(phx_server s, int64_t delta);

namespace {

// Calls that need the instance's device part: refused while a server has evicted it (or has
// not yet admitted it); the server re-creates it on the instance's next request.
int require_resident(phx_instance inst) {
  if (!inst->resident)
    return set_err(PHX_EBUSY, "instance is not on the device (evicted by its server, or not yet admitted): "
                              "submit it to its server again");
  return PHX_OK;
}

template <typename T>
int arena_alloc(phx_instance inst, T** out, size_t count, bool zero = false) {
  size_t bytes = std::max<size_t>(count, 1) * sizeof(T);
  void* p = inst->ctx->arena.alloc(bytes);
  if (!p) return set_err(PHX_ENOMEM, "device arena exhausted (" + std::to_string(bytes) + " bytes requested)");
  inst->blocks.push_back(p);
  inst->bytes += (int64_t)((bytes + 255) & ~(size_t)255);
  if (zero) {
    cudaError_t e = cudaMemsetAsync(p, 0, bytes, inst->ctx->stream);
    if (e != cudaSuccess) return set_err(PHX_ECUDA, cudaGetErrorString(e));
  }
  *out = (T*)p;
  return PHX_OK;
}

template <typename T>
int upload(phx_instance inst, T** out, const std::vector<T>& v) {
  int rc = arena_alloc(inst, out, v.size());
  if (rc) return rc;
  if (!v.empty()) CU(cudaMemcpyAsync(*out, v.data(), v.size() * sizeof(T), cudaMemcpyHostToDevice, inst->ctx->stream));
  return PHX_OK;
}

#define TRY(x)            \
  do {                    \
    int rc_ = (x);        \
    if (rc_) return rc_;  \
  } while (0)

// Device bytes of the arena blocks of `count` elements of `elem` bytes (256-byte granules).
int64_t arena_bytes_of(size_t count, size_t elem) {
  return (int64_t)(((std::max<size_t>(count, 1) * elem) + 255) & ~(size_t)255);
}

// Bytes ensure_precision allocates for one arithmetic (element size s).
int64_t precision_bytes(int64_t n, int64_t m, int64_t nslots, size_t s) {
  const size_t n4 = 4 * (size_t)n;
  return arena_bytes_of(90 * (size_t)m, s) + arena_bytes_of(9 * (size_t)nslots, s) + 6 * arena_bytes_of(n4, s) +
         arena_bytes_of(9 * (size_t)n, s);
}

int ensure_precision_impl(phx_instance inst, bool fp64);

// Allocates the Hessian, PCG and preconditioner buffers of one arithmetic; on failure the
// blocks allocated by this call are released again.
int ensure_precision(phx_instance inst, bool fp64) {
  const size_t nblk = inst->blocks.size();
  const int64_t b0 = inst->bytes;
  const InstDev keep = inst->dev;
  const int rc = ensure_precision_impl(inst, fp64);
  if (rc != PHX_OK) {
    for (size_t k = nblk; k < inst->blocks.size(); ++k) inst->ctx->arena.free(inst->blocks[k]);
    inst->blocks.resize(nblk);
    inst->bytes = b0;
    inst->dev = keep;
  }
  return rc;
}

int ensure_precision_impl(phx_instance inst, bool fp64) {
  InstDev& D = inst->dev;
  const size_t n4 = 4 * (size_t)D.n, m = D.m;
  if (fp64 && !inst->have64) {
    TRY(arena_alloc(inst, &D.Hloc64, 90 * m));
    TRY(arena_alloc(inst, &D.H64, 9 * (size_t)D.nslots, true));
    TRY(arena_alloc(inst, &D.rd, n4, true));
    TRY(arena_alloc(inst, &D.zd, n4, true));
    TRY(arena_alloc(inst, &D.pda, n4, true));
    TRY(arena_alloc(inst, &D.pdb, n4, true));
    TRY(arena_alloc(inst, &D.qd, n4, true));
    TRY(arena_alloc(inst, &D.ed, n4, true));
    TRY(arena_alloc(inst, &D.minvd, 9 * (size_t)D.n, true));
    inst->have64 = true;
  }
  if (!fp64 && !inst->have32) {
    TRY(arena_alloc(inst, &D.Hloc32, 90 * m));
    TRY(arena_alloc(inst, &D.H32, 9 * (size_t)D.nslots, true));
    TRY(arena_alloc(inst, &D.r32, n4, true));
    TRY(arena_alloc(inst, &D.z32, n4, true));
    TRY(arena_alloc(inst, &D.p32a, n4, true));
    TRY(arena_alloc(inst, &D.p32b, n4, true));
    TRY(arena_alloc(inst, &D.q32, n4, true));
    TRY(arena_alloc(inst, &D.e32, n4, true));
    TRY(arena_alloc(inst, &D.minv32, 9 * (size_t)D.n, true));
    inst->have32 = true;
  }
  return PHX_OK;
}

int tiles(int count) { return (count + kTile - 1) / kTile; }

// ---------------------------------------------------------------------------
// batches
// ---------------------------------------------------------------------------
int ensure_batch_cap(phx_context ctx, int num) {
  if (num <= ctx->cap) return PHX_OK;
  int cap = std::max(num, std::max(16, ctx->cap * 2));
  if (ctx->d_inst) cudaFree(ctx->d_inst);
  if (ctx->d_pre) cudaFree(ctx->d_pre);
  if (ctx->d_flags) cudaFree(ctx->d_flags);
  if (ctx->h_flags) cudaFreeHost(ctx->h_flags);
  ctx->d_inst = nullptr; ctx->d_pre = nullptr; ctx->d_flags = nullptr; ctx->h_flags = nullptr;
  CU(cudaMalloc(&ctx->d_inst, sizeof(InstDev) * cap));
  CU(cudaMalloc(&ctx->d_pre, sizeof(int32_t) * (3 * (cap + 1) + 1)));
  CU(cudaMalloc(&ctx->d_flags, sizeof(int32_t) * (8 + cap)));
  CU(cudaMallocHost(&ctx->h_flags, sizeof(int32_t) * (8 + cap)));
  if (ctx->d_corder) cudaFree(ctx->d_corder);
  if (ctx->d_wait) cudaFree(ctx->d_wait);
  ctx->d_corder = nullptr; ctx->d_wait = nullptr;
  CU(cudaMalloc(&ctx->d_corder, sizeof(int32_t) * cap));
  CU(cudaMalloc(&ctx->d_wait, sizeof(int32_t) * wait_size(cap)));
  CU(cudaMemsetAsync(ctx->d_wait, 0, sizeof(int32_t) * kWaitLists, ctx->stream));
  ctx->cap = cap;
  if (!ctx->d_phc) {
    CU(cudaMalloc(&ctx->d_phc, sizeof(int32_t) * 32));
    CU(cudaMemsetAsync(ctx->d_phc, 0, sizeof(int32_t) * 32, ctx->stream));
  }
  return PHX_OK;
}

struct Grids { int tet = 0, node = 0, lob = 0; };

// Uploads the descriptors and tile prefix arrays of a set of instances.
int set_batch(phx_context ctx, const std::vector<phx_instance>& list, BatchDev& B, Grids& G) {
  int num = (int)list.size();
  ctx->batch_owner = nullptr;
  TRY(ensure_batch_cap(ctx, std::max(num, 1)));
  std::vector<InstDev> d(num);
  std::vector<int32_t>& pre = ctx->h_pre;
  pre.assign(3 * (ctx->cap + 1) + 1, 0);
  int32_t* pt = pre.data();
  int32_t* pn = pt + (ctx->cap + 1);
  int32_t* pl = pn + (ctx->cap + 1);
  for (int i = 0; i < num; ++i) {
    d[i] = list[i]->dev;
    pt[i + 1] = pt[i] + tiles(list[i]->dev.m);
    pn[i + 1] = pn[i] + tiles(list[i]->dev.n);
    pl[i + 1] = pl[i] + tiles(list[i]->dev.nlo);
  }
  pre[3 * (ctx->cap + 1)] = num;
  if (num) CU(cudaMemcpyAsync(ctx->d_inst, d.data(), sizeof(InstDev) * num, cudaMemcpyHostToDevice, ctx->stream));
  CU(cudaMemcpyAsync(ctx->d_pre, pre.data(), sizeof(int32_t) * pre.size(), cudaMemcpyHostToDevice, ctx->stream));
  B.num = ctx->d_pre + 3 * (ctx->cap + 1);
  B.pre_tet = ctx->d_pre;
  B.pre_node = ctx->d_pre + (ctx->cap + 1);
  B.pre_lob = ctx->d_pre + 2 * (ctx->cap + 1);
  B.inst = ctx->d_inst;
  B.flags = ctx->d_flags;
  // [0]: active instances (the batch size until the engine has run), [2]: a cluster PCG wait
  // gave up, [4], [5]: instances waiting for each cluster PCG kind
  const int32_t hdr[8] = {num, 0, 0, 0, 0, 0, 0, 0};
  CU(cudaMemcpyAsync(ctx->d_flags, hdr, sizeof(hdr), cudaMemcpyHostToDevice, ctx->stream));
  B.phase_live = ctx->d_phc;
  B.algo_total = ctx->profiling ? ctx->d_algo : nullptr;
  B.cluster_mode = 0;
  const int sms = std::max(1, ctx->num_sms);
  G.tet = std::min(pt[num], sms * 8);
  G.node = std::min(pn[num], sms * 16);
  G.lob = std::min(pl[num], sms * 6);
  return PHX_OK;
}

void do_launch(phx_context ctx, KernelId id, int grid, const BatchDev& B, bool fp64) {
  if (grid <= 0) return;
  if (ctx->profiling) {
    cudaEvent_t a, b;
    if (ctx->pool.size() >= 2) {
      a = ctx->pool.back(); ctx->pool.pop_back();
      b = ctx->pool.back(); ctx->pool.pop_back();
    } else {
      cudaEventCreate(&a);
      cudaEventCreate(&b);
    }
    cudaEventRecord(a, ctx->stream);
    launch(id, grid, ctx->stream, B, fp64);
    cudaEventRecord(b, ctx->stream);
    ctx->evs.push_back({(int)id, a, b});
  } else {
    launch(id, grid, ctx->stream, B, fp64);
  }
  ctx->launches++;
}

int read_flags(phx_context ctx, int num) {
  CU(cudaMemcpyAsync(ctx->h_flags, ctx->d_flags, sizeof(int32_t) * (8 + num), cudaMemcpyDeviceToHost, ctx->stream));
  CU(cudaStreamSynchronize(ctx->stream));
  return PHX_OK;
}

DevOpts make_opts(const phx_options* o, bool dynamic, double dt) {
  DevOpts d{};
  d.qp_solver = o->qp_solver;
  d.min_step_max_count = o->min_step_max_count;
  d.min_impr_max_count = o->min_impr_max_count;
  d.num_max_iters = o->num_max_iters;
  d.try_steepest = o->try_steepest;
  d.ls_num_max_iters = o->ls_num_max_iters;
  d.ls_num_reg_trials = o->ls_num_reg_trials;
  d.lsearch_num_try = o->lsearch_num_try;
  d.precision = o->precision;
  d.precond = o->precond;
  d.max_refine_sweeps = o->precision == PHX_PREC_FP64 ? 1 : std::max(1, o->max_refine_sweeps);
  d.warm_guess = o->warm_guess;
  d.ls_parallel = o->lsearch_parallel;
  d.dynamic = dynamic ? 1 : 0;
  d.tol_max_error = o->tol_max_error;
  d.tol_min_step = o->tol_min_step;
  d.tol_min_impr = o->tol_min_impr;
  d.max_step_size = o->max_step_size;
  d.ls_tol_max_error = o->ls_tol_max_error;
  d.lsearch_alpha = o->lsearch_alpha;
  d.lsearch_type = o->lsearch_type;
  d.lsearch_wolfe1 = o->lsearch_wolfe1;
  d.lsearch_wolfe2 = o->lsearch_wolfe2;
  d.inner_tol = o->inner_tol;
  d.dt = dt;
  d.tol_rel = o->tol_rel;
  d.curv_through = o->negative_curvature == 1 ? 1 : 0;
  return d;
}

int validate_opts(const phx_options* o) {
  if (!o) return set_err(PHX_EINVAL, "options: NULL");
  if (o->precision != PHX_PREC_FP64 && o->precision != PHX_PREC_FP32_REFINE)
    return set_err(PHX_EINVAL, "options: unknown precision");
  if (o->qp_solver != 0 && o->qp_solver != 1) return set_err(PHX_EINVAL, "options: qp_solver must be 0 (Steepest) or 1 (Newton)");
  if (o->lsearch_type < 0 || o->lsearch_type > 4)
    return set_err(PHX_EINVAL, "options: lsearch_type must be 0 (None) .. 4 (WolfeStrong)");
  if (!(o->lsearch_wolfe1 > 0 && o->lsearch_wolfe1 < 1) || !(o->lsearch_wolfe2 > o->lsearch_wolfe1 && o->lsearch_wolfe2 < 1))
    return set_err(PHX_EINVAL, "options: Wolfe constants need 0 < wolfe1 < wolfe2 < 1");
  if (o->ls_num_reg_trials < 1 || o->ls_num_max_iters < 0 || o->num_max_iters < 1)
    return set_err(PHX_EINVAL, "options: non-positive iteration limit");
  if (!(o->lsearch_alpha > 0 && o->lsearch_alpha < 1)) return set_err(PHX_EINVAL, "options: lsearch_alpha out of (0,1)");
  if (o->pcg_chunk < 1 || o->pcg_chunk > 4096) return set_err(PHX_EINVAL, "options: pcg_chunk out of [1,4096]");
  if (!(o->tol_rel >= 0.0)) return set_err(PHX_EINVAL, "options: tol_rel must be >= 0");
  if (o->pcg_cluster < 0 || o->pcg_cluster > 2) return set_err(PHX_EINVAL, "options: pcg_cluster must be 0, 1 or 2");
  if (o->fp64_finish < 0 || o->fp64_finish > 1) return set_err(PHX_EINVAL, "options: fp64_finish must be 0 or 1");
  if (o->lsearch_parallel < 0 || o->lsearch_parallel > kLsK)
    return set_err(PHX_EINVAL, "options: lsearch_parallel out of [0,8]");
  if (o->negative_curvature < 0 || o->negative_curvature > 1)
    return set_err(PHX_EINVAL, "options: negative_curvature must be 0 or 1");
  return PHX_OK;
}

// (A copy from pageable memory to the device is staged by the runtime before the call returns,
// so the local buffer may go at once; nothing waits for the stream.)
int upload_x(phx_instance inst, const double* x3, double* dst) {
  const int n = inst->dev.n;
  std::vector<double> buf(4 * (size_t)n, 0.0);
  for (int v = 0; v < n; ++v)
    for (int c = 0; c < 3; ++c) buf[4 * (size_t)v + c] = x3[3 * (size_t)v + c];
  CU(cudaMemcpyAsync(dst, buf.data(), buf.size() * sizeof(double), cudaMemcpyHostToDevice, inst->ctx->stream));
  return PHX_OK;
}

int download_x(phx_instance inst, const double* src, double* x3) {
  const int n = inst->dev.n;
  std::vector<double> buf(4 * (size_t)n);
  CU(cudaMemcpyAsync(buf.data(), src, buf.size() * sizeof(double), cudaMemcpyDeviceToHost, inst->ctx->stream));
  CU(cudaStreamSynchronize(inst->ctx->stream));
  for (int v = 0; v < n; ++v)
    for (int c = 0; c < 3; ++c) x3[3 * (size_t)v + c] = buf[4 * (size_t)v + c];
  return PHX_OK;
}

int reset_state(phx_instance inst, int phase, int nofix, double shift) {
  NState s{};
  s.phase = phase;
  s.nofix = nofix;
  s.shift = shift;
  s.opt0 = -1.0;
  s.stage = inst->stage;
  CU(cudaMemcpyAsync(inst->d_st, &s, sizeof(NState), cudaMemcpyHostToDevice, inst->ctx->stream));
  return PHX_OK;
}

int read_state(phx_instance inst, NState* s) {
  CU(cudaMemcpyAsync(s, inst->d_st, sizeof(NState), cudaMemcpyDeviceToHost, inst->ctx->stream));
  CU(cudaStreamSynchronize(inst->ctx->stream));
  inst->stage = s->stage;  // the boundary conditions keep their stage after a solve
  return PHX_OK;
}

// The states of a batch (and, where x is given, its positions) copied to the host with one
// synchronisation: device-to-host copies into the context's pinned landing area, then unpacked.
int read_batch(phx_context ctx, const std::vector<phx_instance>& list, std::vector<NState>& st, double* const* x) {
  const size_t k = list.size();
  std::vector<size_t> off(k + 1, 0);
  size_t s_bytes = ((k * sizeof(NState)) + 255) & ~(size_t)255;
  off[0] = s_bytes;
  for (size_t i = 0; i < k; ++i)
    off[i + 1] = off[i] + ((x && x[i]) ? ((4 * (size_t)list[i]->dev.n * sizeof(double) + 255) & ~(size_t)255) : 0);
  const size_t need = off[k];
  if (need > ctx->down_cap) {
    if (ctx->down) cudaFreeHost(ctx->down);
    ctx->down = nullptr;
    ctx->down_cap = 0;
    const size_t cap = (need + ((size_t)1 << 20) - 1) & ~(((size_t)1 << 20) - 1);
    if (cudaMallocHost(&ctx->down, cap) != cudaSuccess) {
      cudaGetLastError();
      ctx->down = nullptr;
      // pageable fallback: one instance at a time
      st.resize(k);
      for (size_t i = 0; i < k; ++i) {
        TRY(read_state(list[i], &st[i]));
        if (x && x[i]) TRY(download_x(list[i], list[i]->dev.x, x[i]));
      }
      return PHX_OK;
    }
    ctx->down_cap = cap;
  }
  NState* hs = reinterpret_cast<NState*>(ctx->down);
  for (size_t i = 0; i < k; ++i) {
    CU(cudaMemcpyAsync(hs + i, list[i]->d_st, sizeof(NState), cudaMemcpyDeviceToHost, ctx->stream));
    if (x && x[i])
      CU(cudaMemcpyAsync(ctx->down + off[i], list[i]->dev.x, 4 * (size_t)list[i]->dev.n * sizeof(double),
                         cudaMemcpyDeviceToHost, ctx->stream));
  }
  CU(cudaStreamSynchronize(ctx->stream));
  st.resize(k);
  for (size_t i = 0; i < k; ++i) {
    st[i] = hs[i];
    list[i]->stage = st[i].stage;  // the boundary conditions keep their stage after a solve
    if (x && x[i]) {
      const double* b = reinterpret_cast<const double*>(ctx->down + off[i]);
      for (int v = 0; v < list[i]->dev.n; ++v)
        for (int c = 0; c < 3; ++c) x[i][3 * (size_t)v + c] = b[4 * (size_t)v + c];
    }
  }
  return PHX_OK;
}

void fill_report(const NState& s, bool step, double seconds, phx_report* r) {
  if (!r) return;
  r->result = step ? s.step_result : s.result;
  r->iterations = s.it;
  r->bisections = s.total_bis;
  r->reg_trials = s.total_reg;
  r->pcg_iterations = s.pcg_total;
  r->refine_sweeps = s.total_sweeps;
  r->status = s.error ? PHX_ETIMEOUT : PHX_OK;
  r->obj = s.obj;
  r->opt = s.opt;
  r->opt0 = s.opt0;
  r->seconds = seconds;
  r->hessian_evals = s.hess_count;
  r->fp64_iterations = 0;
  r->pcg_slices = s.pcg_slices;
}

// Report of a static solve that an FP64 finish continued: counts of both parts, the
// result, energy and gradient of the finish, the starting gradient of the first.
void fill_report_finished(const NState& a, const NState& b, double seconds, phx_report* r) {
  if (!r) return;
  fill_report(b, false, seconds, r);
  r->iterations += a.it;
  r->bisections += a.total_bis;
  r->reg_trials += a.total_reg;
  r->pcg_iterations += a.pcg_total;
  r->refine_sweeps += a.total_sweeps;
  r->hessian_evals += a.hess_count;
  r->pcg_slices += a.pcg_slices;
  r->opt0 = a.opt0;
  r->fp64_iterations = b.it;
  if (a.error) r->status = PHX_ETIMEOUT;
}

int ensure_engine(phx_context ctx) {
  if (!ctx->d_bar) CU(cudaMalloc(&ctx->d_bar, 2 * sizeof(GridBar)));
  if (!ctx->d_cfg) {
    CU(cudaMalloc(&ctx->d_cfg, 4 * sizeof(int32_t)));
    CU(cudaMemsetAsync(ctx->d_cfg, 0, 4 * sizeof(int32_t), ctx->stream));
  }
  if (ctx->act_cap < ctx->cap) {
    if (ctx->d_act) cudaFree(ctx->d_act);
    ctx->d_act = nullptr;
    CU(cudaMalloc(&ctx->d_act, sizeof(int32_t) * (4 + ctx->cap + 4 * (ctx->cap + 1))));
    ctx->act_cap = ctx->cap;
  }
  if (ctx->profiling && !ctx->d_stage) {
    CU(cudaMalloc(&ctx->d_stage, sizeof(unsigned long long) * 32));
    CU(cudaMemsetAsync(ctx->d_stage, 0, sizeof(unsigned long long) * 32, ctx->stream));
  }
  return PHX_OK;
}

// A pair of timing events from the pool, the first recorded now on the library stream.
int profile_events(phx_context ctx, cudaEvent_t* a, cudaEvent_t* b) {
  if (ctx->pool.size() >= 2) {
    *a = ctx->pool.back(); ctx->pool.pop_back();
    *b = ctx->pool.back(); ctx->pool.pop_back();
  } else {
    CU(cudaEventCreate(a));
    CU(cudaEventCreate(b));
  }
  CU(cudaEventRecord(*a, ctx->stream));
  return PHX_OK;
}

int engine_grid_of(phx_context ctx, bool fp64, int* grid) {
  int& g = ctx->egrid[fp64 ? 1 : 0];
  if (g == 0) g = engine_grid(fp64, ctx->num_sms);
  if (g <= 0) return set_err(PHX_ECUDA, "engine kernel cannot be made resident");
  *grid = g;
  return PHX_OK;
}

EngineArgs engine_args(phx_context ctx, const phx_launch_settings& S, int pcg_chunk) {
  EngineArgs A{};
  A.bar = ctx->d_bar;
  A.act = ctx->d_act;
  A.stage_ns = ctx->profiling ? ctx->d_stage : nullptr;
  A.cap = ctx->cap;
  A.rounds = S.rounds;
  A.pcg_chunk = pcg_chunk;
  A.wait_rounds = S.wait_rounds;
  A.wait_share = S.wait_share;
  A.slice_share = S.slice_share;
  A.slice_min = S.slice_min;
  A.wait_limit = ctx->wait_limit;
  A.unmet_tag = ctx->unmet_tag;
  A.cfg = ctx->d_cfg;
  A.corder = ctx->d_corder;
  A.ccount = ctx->ccount;
  A.wait = ctx->d_wait;
  return A;
}

// One cooperative launch of the engine: up to `rounds` Newton rounds over the batch.
int run_engine(phx_context ctx, const BatchDev& B, int num, bool fp64, const phx_launch_settings& S, int pcg_chunk) {
  TRY(ensure_engine(ctx));
  int grid;
  TRY(engine_grid_of(ctx, fp64, &grid));
  const EngineArgs A = engine_args(ctx, S, pcg_chunk);
  CU(launch_prep(ctx->stream, B, A, grid));
  cudaEvent_t a = nullptr, b = nullptr;
  if (ctx->profiling) TRY(profile_events(ctx, &a, &b));
  CU(launch_engine(fp64, grid, ctx->stream, B, A));
  ctx->launches += 2;
  if (ctx->profiling) {
    cudaEventRecord(b, ctx->stream);
    ctx->evs.push_back({(int)K_ENGINE, a, b});
  }
  GridBar hb[2];
  CU(cudaMemcpyAsync(hb, ctx->d_bar, 2 * sizeof(GridBar), cudaMemcpyDeviceToHost, ctx->stream));
  TRY(read_flags(ctx, num));
  if (hb[0].err || hb[1].err)
    return set_err(PHX_ETIMEOUT, "engine grid barrier timed out (stage " +
                                     std::to_string(hb[1].err ? hb[1].stage : hb[0].stage) + ")");
  return PHX_OK;
}

// Uploads the batch positions of the instances whose PCG runs per cluster, largest first.
// Uploads the batch positions of the instances whose PCG runs per cluster, largest first (the
// order in which the engine lists them for the cluster kernels).
int set_cluster_list(phx_context ctx, const std::vector<phx_instance>& list, int* count) {
  std::vector<int32_t> ids;
  for (int i = 0; i < (int)list.size(); ++i)
    if (list[i]->dev.pcg_cluster) ids.push_back(i);
  std::stable_sort(ids.begin(), ids.end(), [&](int a, int b) { return list[a]->dev.nslots > list[b]->dev.nslots; });
  *count = (int)ids.size();
  ctx->ccount = (int)ids.size();
  for (int k = 0; k < 4; ++k) ctx->ckind_count[k] = 0;
  for (int id : ids) ctx->ckind_count[list[id]->dev.pcg_cluster]++;
  if (!ids.empty())  // pageable source: copied before the call returns
    CU(cudaMemcpyAsync(ctx->d_corder, ids.data(), sizeof(int32_t) * ids.size(), cudaMemcpyHostToDevice, ctx->stream));
  return PHX_OK;
}

// Clusters to launch for `waiting` instances of PCG kind `kind`: one per instance, at most as
// many as are resident at once (each cluster takes instances from the list until none is left).
int cluster_count(phx_context ctx, int kind, int waiting) {
  if (ctx->gmax[kind] < 0) ctx->gmax[kind] = max_active_clusters(kind);
  return ctx->gmax[kind] > 0 ? std::min(waiting, ctx->gmax[kind]) : waiting;
}

// The whole-GPU PCG of the listed kind-3 instances, until each has left its PCG: blocks of
// kGpcgBlock iterations, the host reading the count left between blocks.  Profiling puts a
// pair of events around every kernel.
constexpr int kGpcgBlock = 16;

int run_gpcg(phx_context ctx, const BatchDev& B, const phx_launch_settings& S, int pcg_chunk) {
  if (ctx->ggrid == 0) ctx->ggrid = gpcg_grid(ctx->num_sms);
  const EngineArgs A = engine_args(ctx, S, pcg_chunk);
  for (int64_t it = 0;; it += kGpcgBlock) {
    for (int k = 0; k < kGpcgBlock; ++k) {
      if (ctx->profiling) {
        cudaEvent_t ev[4];
        TRY(profile_events(ctx, &ev[0], &ev[1]));  // records ev[0]
        TRY(profile_events(ctx, &ev[2], &ev[3]));  // records ev[2]: the pair is recorded again below
        CU(launch_gpcg(ctx->stream, B, A, ctx->ggrid, 1, ev));
        ctx->evs.push_back({(int)K_PCG_A, ev[0], ev[1]});
        ctx->evs.push_back({(int)K_PCG_B, ev[2], ev[3]});
      } else {
        CU(launch_gpcg(ctx->stream, B, A, ctx->ggrid, 1));
      }
      ctx->launches += 2;
    }
    int32_t left = 0;
    CU(cudaMemcpyAsync(&left, ctx->d_wait + kWaitLeft, sizeof(int32_t), cudaMemcpyDeviceToHost, ctx->stream));
    CU(cudaStreamSynchronize(ctx->stream));
    if (left <= 0) return PHX_OK;
    if (it >= (int64_t)1 << 20) return set_err(PHX_ETIMEOUT, "whole-GPU PCG did not finish");
  }
}

// One step of the device engine: engine rounds, then (if any) the per-cluster PCG solves.
// PCG placement: FP32 instances small enough iterate inside wide clusters (measured
// faster than the grid-wide PCG both while many instances are active and in the tail);
// the rest iterate on the whole GPU, with one-chunk tiles while few small instances
// remain so that a lone instance spreads over more SMs.
int run_step(phx_context ctx, const BatchDev& B0, int num, bool fp64, int pcg_chunk, int ccount,
             const phx_launch_settings& S) {
  BatchDev B = B0;
  B.cluster_mode = ccount > 0 ? 1 : 0;
  // (each instance's PCG tile width is its own: one-chunk tiles for small instances, which
  // then spread over many CTAs, four-chunk tiles for large ones)
  TRY(run_engine(ctx, B, num, fp64, S, pcg_chunk));
  if (ctx->h_flags[2]) return set_err(PHX_ETIMEOUT, "cluster PCG reduction wait timed out");
  if (B.cluster_mode && ctx->h_flags[0] > 0 && ctx->h_flags[1] > 0) {
    cudaEvent_t a = nullptr, b = nullptr;
    if (ctx->profiling) TRY(profile_events(ctx, &a, &b));
    // the engine listed the waiting instances of each kind, largest first; the clusters take
    // them from the list in that order
    for (int kind = 1; kind <= 2; ++kind) {
      const int nw = ctx->h_flags[3 + kind];
      if (nw == 0) continue;
      CU(launch_pcg_cluster(ctx->stream, B, ctx->d_wait, ctx->cap, cluster_count(ctx, kind, nw), kind, S.slice_share,
                            S.slice_min));
      ctx->launches++;
    }
    if (ctx->h_flags[6] > 0) TRY(run_gpcg(ctx, B, S, pcg_chunk));
    if (ctx->profiling) {
      cudaEventRecord(b, ctx->stream);
      ctx->evs.push_back({(int)K_PCG_CLUSTER, a, b});
    }
  }
  return PHX_OK;
}

// The solve loop as graph launches: each launch runs up to kGraphPasses passes of k_prep, the
// engine, the cluster PCG kernels and k_loop_end on the device, with no host step between them;
// the host checks the outcome (and the time limit) between launches.
constexpr int kGraphPasses = 256;

int run_graph(phx_context ctx, const BatchDev& B0, int num, bool fp64, int pcg_chunk,
              const phx_launch_settings& S, clk::time_point t0) {
  TRY(ensure_engine(ctx));
  int grid;
  TRY(engine_grid_of(ctx, fp64, &grid));
  BatchDev B = B0;
  B.cluster_mode = ctx->ccount > 0 ? 1 : 0;
  const EngineArgs A = engine_args(ctx, S, pcg_chunk);
  int clusters[2] = {0, 0};
  for (int kind = 1; kind <= 2; ++kind)
    if (B.cluster_mode && ctx->ckind_count[kind] > 0) clusters[kind - 1] = cluster_count(ctx, kind, ctx->ckind_count[kind]);
  if (ctx->ggrid == 0) ctx->ggrid = gpcg_grid(ctx->num_sms);
  const int gpcg = (B.cluster_mode && ctx->ckind_count[3] > 0) ? ctx->ggrid : 0;
  // the graph holds its kernels' arguments: rebuilt when any of them changes
  std::string key;
  auto put = [&](const void* p, size_t n) { key.append(static_cast<const char*>(p), n); };
  put(&fp64, sizeof(fp64)); put(&grid, sizeof(grid)); put(&B, sizeof(B)); put(&A, sizeof(A));
  put(clusters, sizeof(clusters)); put(&gpcg, sizeof(gpcg));
  if (!ctx->gexec || key != ctx->gkey) {
    if (ctx->gexec) cudaGraphExecDestroy(ctx->gexec);
    if (ctx->graph) cudaGraphDestroy(ctx->graph);
    ctx->gexec = nullptr;
    ctx->graph = nullptr;
    ctx->gkey.clear();
    CU(build_solve_graph(fp64, grid, B, A, clusters, gpcg, ctx->d_cfg + 1, kGraphPasses, &ctx->graph,
                         &ctx->gexec));
    ctx->gkey = key;
  }
  const int per_pass = 3 + (clusters[0] > 0) + (clusters[1] > 0) + (gpcg > 0);
  for (;;) {
    CU(cudaMemsetAsync(ctx->d_cfg + 1, 0, 2 * sizeof(int32_t), ctx->stream));
    CU(cudaGraphLaunch(ctx->gexec, ctx->stream));
    GridBar hb[2];
    int32_t passes[2] = {0, 0};
    CU(cudaMemcpyAsync(hb, ctx->d_bar, 2 * sizeof(GridBar), cudaMemcpyDeviceToHost, ctx->stream));
    CU(cudaMemcpyAsync(passes, ctx->d_cfg + 1, 2 * sizeof(int32_t), cudaMemcpyDeviceToHost, ctx->stream));
    TRY(read_flags(ctx, num));
    ctx->launches += (int64_t)passes[0] * per_pass + 3 * (int64_t)passes[1];
    if (hb[0].err || hb[1].err)
      return set_err(PHX_ETIMEOUT, "engine grid barrier timed out (stage " +
                                       std::to_string(hb[1].err ? hb[1].stage : hb[0].stage) + ")");
    if (ctx->h_flags[2]) return set_err(PHX_ETIMEOUT, "cluster PCG reduction wait timed out");
    if (ctx->h_flags[0] == 0) return PHX_OK;
    if (std::chrono::duration<double>(clk::now() - t0).count() > kSolveTimeLimit)
      return set_err(PHX_ETIMEOUT, "solver did not finish within " + std::to_string(kSolveTimeLimit) + " s");
  }
}

// The PCG kind of FP32 instances above the cluster size for this run: the whole-GPU kernels
// (kind 3) or the engine's stages (kind 0); start_solve marks them 3 and sets grid_eligible.
void apply_pcg_grid(const std::vector<phx_instance>& list, const phx_launch_settings& S) {
  for (auto* in : list)
    if (in->grid_eligible) in->dev.pcg_cluster = S.pcg_grid ? 3 : 0;
}

// Batch mix key of the tuned-settings cache: precision, then instances per power-of-two
// node-count bucket.
std::string mix_key(const std::vector<phx_instance>& list, bool fp64) {
  std::map<int, int> buckets;
  for (auto* in : list) {
    int b = 0;
    while ((1 << (b + 1)) <= in->dev.n && b < 30) ++b;
    buckets[b]++;
  }
  std::string k = fp64 ? "f64" : "f32";
  for (auto& kv : buckets) k += "|" + std::to_string(kv.first) + ":" + std::to_string(kv.second);
  return k;
}

// Runs a set of instances (states already reset to PH_START) until all are done, with the
// given launch settings, else those tuned for the batch's mix, else the context's defaults.
int run_to_completion(phx_context ctx, const std::vector<phx_instance>& list, bool fp64, int pcg_chunk,
                      const phx_launch_settings* force = nullptr) {
  phx_launch_settings S = ctx->launch;
  if (force) {
    S = *force;
  } else if (!ctx->tuned.empty()) {
    auto it = ctx->tuned.find(mix_key(list, fp64));
    if (it != ctx->tuned.end()) S = it->second;
  }
  apply_pcg_grid(list, S);
  BatchDev B{};
  Grids G;
  TRY(set_batch(ctx, list, B, G));
  int ccount = 0;
  TRY(set_cluster_list(ctx, list, &ccount));
  const int num = (int)list.size();
  const auto t0 = clk::now();
  int active = num;
  // per-launch timing events need the host between launches: profiling runs the host loop
  if (S.graph && !ctx->profiling) return run_graph(ctx, B, num, fp64, pcg_chunk, S, t0);
  for (int64_t r = 0;; ++r) {
    TRY(run_step(ctx, B, num, fp64, pcg_chunk, ccount, S));
    active = ctx->h_flags[0];
    if (active == 0) return PHX_OK;
    if (std::chrono::duration<double>(clk::now() - t0).count() > kSolveTimeLimit)
      return set_err(PHX_ETIMEOUT, "solver did not finish within " + std::to_string(kSolveTimeLimit) + " s");
  }
}

// Algorithmic bytes one launch of each kernel moves for this instance: every input it
// must read and every output it must write, once (padding, re-reads and caches excluded).
void set_algo_bytes(InstDev& D, bool fp64) {
  const double s = fp64 ? 8.0 : 4.0, n = D.n, m = D.m, nlo = D.nlo, nfull = 2.0 * D.nlo - D.n, N = 3.0 * D.n;
  for (int k = 0; k < 16; ++k) D.algo[k] = 0.0;
  D.algo[K_ELEM_EG] = 16 * m + 96 * m + m + 8 * N + 96 * m + 8 * m;
  D.algo[K_GATHER] = 96 * m + 16 * m + 4 * (n + 1) + n + 3 * 8 * N;
  D.algo[K_ELEM_HESS] = 16 * m + 12 * s * m + m + 8 * N + 90 * s * m;
  D.algo[K_ASSEMBLE] = 90 * s * m + 40 * m + 4 * (nlo + 1) + 16 * nlo + n + 9 * s * nfull;
  D.algo[K_JACOBI] = 18 * s * n;
  D.algo[K_LINSETUP] = 4 * 8 * N;
  D.algo[K_RESID] = nfull * (9 * s + 4) + 3 * 8 * N + 9 * s * n + 4 * s * N;
  D.algo[K_PCG_A] = nfull * (9 * s + 4) + 4 * s * N;
  D.algo[K_PCG_B] = 7 * s * N + 9 * s * n;
  D.algo[K_ACCUM] = s * N + 2 * 8 * N;
}

int start_solve(phx_instance inst, const phx_options* o, bool dynamic, double dt, int max_iters_override) {
  TRY(validate_opts(o));
  const bool fp64 = o->precision == PHX_PREC_FP64;
  TRY(ensure_precision(inst, fp64));
  DevOpts d = make_opts(o, dynamic, dt);
  if (max_iters_override > 0) d.num_max_iters = max_iters_override;
  d.num_stages = inst->num_stages;
  d.stage_values = inst->stage_values ? 1 : 0;
  set_algo_bytes(inst->dev, fp64);
  // the cluster PCG serves the FP32 path: FP64 arithmetic is slow on this part and needs
  // every SM, so FP64 solves iterate on the whole GPU
  // larger FP32 instances iterate in the whole-GPU PCG kernels (kind 3)
  // (kind 3 becomes 0, the engine's PCG stages, unless the launch settings pick the grid kernels)
  inst->dev.pcg_cluster = (o->pcg_cluster < 1 || o->pcg_cluster > 2 || fp64) ? 0
                          : inst->dev.n <= kClusterMaxNodes                 ? o->pcg_cluster
                                                                              : 3;
  inst->grid_eligible = inst->dev.pcg_cluster == 3;
  CU(cudaMemcpyAsync(inst->d_opts, &d, sizeof(DevOpts), cudaMemcpyHostToDevice, inst->ctx->stream));
  TRY(reset_state(inst, PH_START, 0, 0.0));
  return PHX_OK;
}

// FP32 solves that stall within kFinishFactor of their tolerance, or after reducing the
// gradient a hundredfold: the FP32-stored Hessian
// makes Newton converge linearly there, and near an equilibrium the energy decrease of
// a step can fall below the FP64 energy comparison's resolution before the gradient
// meets a tolerance taken relative to a small starting gradient (warm re-solves).
constexpr double kFinishFactor = 1e3;

bool wants_fp64_finish(const phx_options* o, const NState& s) {
  if (!o->fp64_finish || o->precision != PHX_PREC_FP32_REFINE || s.error) return false;
  const bool stalled = s.result == OS_NONDESC || s.result == OS_MINIMPR || s.result == OS_MINSTEP ||
                       s.result == OS_MAXITER;
  // close to the tolerance, or well on the way there (diverged solves stay failures)
  return stalled && std::isfinite(s.opt) && (s.opt <= kFinishFactor * s.tol_eff || s.opt <= 1e-2 * s.opt0);
}

// Continues the listed FP32 solves in FP64 from their restart points (the last accepted
// iterate with ||g|| above kBackFactor x tolerance), to the same absolute tolerance, with
// the FP32 solve's PCG budget per Newton step in one solve.
int finish_fp64(phx_context ctx, const std::vector<phx_instance>& list, const phx_options* o,
                const std::vector<NState>& first, std::vector<NState>* second) {
  for (size_t k = 0; k < list.size(); ++k) {
    // restart from the last accepted iterate whose gradient was well above the tolerance:
    // the iterate FP32 stalled at can sit where the energy comparison no longer resolves a
    // step, which an exact Newton step from the restart point jumps over
    InstDev& D = list[k]->dev;
    if (!(first[k].opt > kBackFactor * first[k].tol_eff))  // else the last iterate itself is the restart point
      CU(cudaMemcpyAsync(D.x, D.xback, 4 * sizeof(double) * (size_t)D.n, cudaMemcpyDeviceToDevice, ctx->stream));
    phx_options f = *o;
    f.precision = PHX_PREC_FP64;
    f.tol_rel = 0.0;
    f.tol_max_error = first[k].tol_eff;
    f.ls_num_max_iters = o->ls_num_max_iters * std::max(1, o->max_refine_sweeps);
    TRY(start_solve(list[k], &f, false, 0.0, 0));
  }
  TRY(run_to_completion(ctx, list, true, o->pcg_chunk));
  second->resize(list.size());
  for (size_t k = 0; k < list.size(); ++k) TRY(read_state(list[k], &(*second)[k]));
  return PHX_OK;
}

}  // namespace

// ===========================================================================
// C ABI
// ===========================================================================
extern "C" {

int phx_version(void) { return 10100; }

const char* phx_last_error(void) { return g_err.c_str(); }

void phx_default_options(phx_options* o) {
  if (!o) return;
  std::memset(o, 0, sizeof(*o));
  o->qp_solver = 1;
  o->tol_max_error = 1e-6;
  o->tol_min_step = 1e-5;
  o->min_step_max_count = 3;
  o->tol_min_impr = 1e-9;
  o->min_impr_max_count = 3;
  o->num_max_iters = 100;
  o->try_steepest = 1;
  o->max_step_size = 1000;
  o->ls_solver = 1;
  o->ls_num_max_iters = 1000;
  o->ls_tol_max_error = 1e-9;
  o->ls_num_reg_trials = 10;
  o->lsearch_type = 1;
  o->lsearch_alpha = 0.5;
  o->lsearch_num_try = 32;
  o->lsearch_wolfe1 = 1e-4;
  o->lsearch_wolfe2 = 0.9;
  o->precision = PHX_PREC_FP64;
  o->precond = 1;
  o->inner_tol = 1e-4;
  o->max_refine_sweeps = 12;
  o->warm_guess = 1;
  o->pcg_chunk = 32;
  o->tol_rel = 0.0;
  o->pcg_cluster = 1;
  o->fp64_finish = 1;
  o->lsearch_parallel = 8;
}

int phx_context_create(int32_t device, int64_t arena_bytes, phx_context* out) {
  if (!out) return set_err(PHX_EINVAL, "out is NULL");
  *out = nullptr;
  int count = 0;
  CU(cudaGetDeviceCount(&count));
  if (device < 0 || device >= count) return set_err(PHX_EINVAL, "no such CUDA device");
  CU(cudaSetDevice(device));
  auto* ctx = new phx_context_s();
  ctx->device = device;
  cudaError_t e = cudaDeviceGetAttribute(&ctx->num_sms, cudaDevAttrMultiProcessorCount, device);
  if (e == cudaSuccess) e = cudaStreamCreateWithFlags(&ctx->stream, cudaStreamNonBlocking);
  if (e == cudaSuccess) e = setup_kernel_attributes();
  size_t fr = 0, tot = 0;
  if (e == cudaSuccess) e = cudaMemGetInfo(&fr, &tot);
  if (e == cudaSuccess) {
    size_t want = arena_bytes > 0 ? (size_t)arena_bytes : fr / 4;
    e = ctx->arena.init(want);
  }
  if (e != cudaSuccess) {
    if (ctx->stream) cudaStreamDestroy(ctx->stream);
    delete ctx;
    return set_err(PHX_ECUDA, std::string("context: ") + cudaGetErrorString(e));
  }
  *out = ctx;
  return PHX_OK;
}

int phx_context_destroy(phx_context ctx) {
  if (!ctx) return PHX_OK;
  cudaSetDevice(ctx->device);
  cudaStreamSynchronize(ctx->stream);
  for (auto& ev : ctx->evs) { cudaEventDestroy(ev.a); cudaEventDestroy(ev.b); }
  for (auto& ev : ctx->pool) cudaEventDestroy(ev);
  if (ctx->d_inst) cudaFree(ctx->d_inst);
  if (ctx->d_pre) cudaFree(ctx->d_pre);
  if (ctx->d_flags) cudaFree(ctx->d_flags);
  if (ctx->h_flags) cudaFreeHost(ctx->h_flags);
  if (ctx->d_algo) cudaFree(ctx->d_algo);
  if (ctx->d_bar) cudaFree(ctx->d_bar);
  if (ctx->d_phc) cudaFree(ctx->d_phc);
  if (ctx->d_act) cudaFree(ctx->d_act);
  if (ctx->d_stage) cudaFree(ctx->d_stage);
  if (ctx->d_corder) cudaFree(ctx->d_corder);
  if (ctx->d_wait) cudaFree(ctx->d_wait);
  if (ctx->d_cfg) cudaFree(ctx->d_cfg);
  if (ctx->gexec) cudaGraphExecDestroy(ctx->gexec);
  if (ctx->graph) cudaGraphDestroy(ctx->graph);
  if (ctx->stage) cudaFreeHost(ctx->stage);
  if (ctx->stage_ev) cudaEventDestroy(ctx->stage_ev);
  if (ctx->down) cudaFreeHost(ctx->down);
  for (auto& ev : ctx->marks)
    if (ev) cudaEventDestroy(ev);
  ctx->arena.release();
  cudaStreamDestroy(ctx->stream);
  delete ctx;
  return PHX_OK;
}

int phx_debug_unmet_barrier(phx_context ctx, int32_t barrier_tag, int64_t limit_cycles) {
  if (!ctx) return set_err(PHX_EINVAL, "ctx is NULL");
  if (barrier_tag < 0 || barrier_tag > 22) return set_err(PHX_EINVAL, "barrier_tag must be 0 (off) or 1..22");
  if (barrier_tag == 0) {
    ctx->unmet_tag = 0;
    ctx->wait_limit = kBarrierLimit;
    return PHX_OK;
  }
  if (limit_cycles < 1000 || limit_cycles > kBarrierLimit)
    return set_err(PHX_EINVAL, "limit_cycles must lie in [1000, 4e9]");
  ctx->unmet_tag = barrier_tag;
  ctx->wait_limit = limit_cycles;
  return PHX_OK;
}

int phx_context_memory(phx_context ctx, int64_t* used, int64_t* cap) {
  if (!ctx) return set_err(PHX_EINVAL, "ctx is NULL");
  if (used) *used = (int64_t)ctx->arena.used;
  if (cap) *cap = (int64_t)ctx->arena.cap;
  return PHX_OK;
}

int phx_instance_destroy(phx_instance inst) {
  if (!inst) return PHX_OK;
  if (inst->in_server) return set_err(PHX_EBUSY, "instance is admitted to a server");
  if (inst->owner) server_forget(inst->owner, inst);  // its bytes leave the server's budget
  cudaStreamSynchronize(inst->ctx->stream);
  for (void* p : inst->blocks) inst->ctx->arena.free(p);
  delete inst;
  return PHX_OK;
}

namespace {

// Host part of creating an instance: validation, the pattern, the rest data and the loads
// (no CUDA call, so instances can be built on several host threads at once).
bool instance_build_host(const phx_mesh* mesh, phx_instance_s* inst, std::string& err) {
  MeshIn in;
  in.n = mesh->num_nodes;
  in.m = mesh->num_tets;
  in.X0 = mesh->X0;
  in.T = mesh->tets;
  in.lame = mesh->lame;
  in.rho = mesh->rho;
  in.model = mesh->model;
  in.fixed = mesh->fixed;
  in.force = mesh->force;
  for (int c = 0; c < 3; ++c) in.gravity[c] = mesh->gravity[c];
  in.soft_k = mesh->soft_k;
  in.soft_target = mesh->soft_target;
  if (!build_pattern(in, inst->hp, err)) return false;
  for (int c = 0; c < 3; ++c) inst->gravity[c] = mesh->gravity[c];
  if (mesh->force) inst->force.assign(mesh->force, mesh->force + 3 * (size_t)in.n);
  return true;
}

// Device bytes instance_setup_device allocates for a built host part, plus the buffers of
// the arithmetic(s) asked for (the serving admission's estimate; equal to the instance's
// bytes after the set-up, which a GPU test checks).
int64_t device_bytes(const HostPattern& hp, bool fp32, bool fp64) {
  int64_t b = (int64_t)base_layout(hp).total;
  if (fp32) b += precision_bytes(hp.n, hp.m, hp.nslots, 4);
  if (fp64) b += precision_bytes(hp.n, hp.m, hp.nslots, 8);
  return b;
}

// Releases an instance's device part (arena blocks) and keeps its host part.
int instance_free_device(phx_instance inst) {
  cudaError_t e = cudaStreamSynchronize(inst->ctx->stream);
  for (void* p : inst->blocks) inst->ctx->arena.free(p);
  inst->blocks.clear();
  inst->dev = InstDev{};
  inst->d_st = nullptr;
  inst->d_opts = nullptr;
  inst->have32 = inst->have64 = false;
  inst->bytes = 0;
  inst->resident = false;
  if (e != cudaSuccess) return set_err(PHX_ECUDA, cudaGetErrorString(e));
  return PHX_OK;
}

// Device part: arena allocations and uploads on the context stream (the caller
// synchronises).  On failure the instance is destroyed, or with keep_on_fail only its
// device part is released.
// Device part from an already packed upload (base_layout / pack_base): one arena block, one
// copy from `staged` (the context's pinned staging, or pageable memory) and one memset, on the
// context stream (the caller synchronises).  On failure the instance is
// destroyed, or with keep_on_fail only its device part is freed.
int setup_from_stage(phx_context ctx, phx_instance_s* inst, const BaseLayout& L, const char* staged,
                     bool keep_on_fail) {
  HostPattern& hp = inst->hp;
  InstDev& D = inst->dev;
  D.n = hp.n; D.m = hp.m; D.nlo = hp.nlo; D.nchunks = hp.nchunks; D.nslots = hp.nslots;
  inst->resident = true;
  auto fail = [&](int rc) {
    if (keep_on_fail) instance_free_device(inst);
    else phx_instance_destroy(inst);
    return rc;
  };
  char* base = nullptr;
  int rc = arena_alloc(inst, &base, L.total);
  if (rc) return fail(rc);
  cudaError_t e = cudaMemcpyAsync(base, staged, L.upload_end, cudaMemcpyHostToDevice, ctx->stream);
  if (e == cudaSuccess) e = cudaMemsetAsync(base + L.upload_end, 0, L.zero_end - L.upload_end, ctx->stream);
  if (e != cudaSuccess) return fail(set_err(PHX_ECUDA, cudaGetErrorString(e)));
  auto at = [&](const BaseLayout::Part& p) { return base + p.off; };
  D.tets = reinterpret_cast<const int32_t*>(at(L.tets));
  D.rest64 = reinterpret_cast<const double*>(at(L.rest64));
  D.rest32 = reinterpret_cast<const float*>(at(L.rest32));
  D.tile_nptr = reinterpret_cast<const int32_t*>(at(L.tile_nptr));
  D.tile_nodes = reinterpret_cast<const int32_t*>(at(L.tile_nodes));
  D.tet_loc = reinterpret_cast<const uint16_t*>(at(L.tet_loc));
  D.model = reinterpret_cast<const uint8_t*>(at(L.model));
  D.chunk_off = reinterpret_cast<const int32_t*>(at(L.chunk_off));
  D.slot_col = reinterpret_cast<const int32_t*>(at(L.slot_col));
  D.diag_slot = reinterpret_cast<const int32_t*>(at(L.diag_slot));
  D.lo_rc = reinterpret_cast<const int32_t*>(at(L.lo_rc));
  D.lo_slot = reinterpret_cast<const int32_t*>(at(L.lo_slot));
  D.up_slot = reinterpret_cast<const int32_t*>(at(L.up_slot));
  D.seg_ptr = reinterpret_cast<const int32_t*>(at(L.seg_ptr));
  D.seg_c = reinterpret_cast<const int32_t*>(at(L.seg_c));
  D.nseg_ptr = reinterpret_cast<const int32_t*>(at(L.nseg_ptr));
  D.nseg_c = reinterpret_cast<const int32_t*>(at(L.nseg_c));
  D.fixmask = reinterpret_cast<const uint8_t*>(at(L.fixmask));
  D.mass = reinterpret_cast<const double*>(at(L.mass));
  D.hlin = reinterpret_cast<double*>(at(L.hlin));
  D.soft = hp.soft.empty() ? nullptr : reinterpret_cast<double*>(at(L.soft));
  D.x = reinterpret_cast<double*>(at(L.x));
  D.xrest = reinterpret_cast<const double*>(at(L.xrest));
  double** vecs[11] = {&D.xs, &D.dx, &D.g, &D.gn, &D.dxprev, &D.x0, &D.v0, &D.v, &D.r64, &D.bvec, &D.xback};
  for (int k = 0; k < 11; ++k) *vecs[k] = reinterpret_cast<double*>(at(L.vec[k]));
  D.counter = reinterpret_cast<uint32_t*>(at(L.counter));
  D.log = reinterpret_cast<double*>(at(L.log));
  inst->d_st = reinterpret_cast<NState*>(at(L.st));
  inst->d_opts = reinterpret_cast<DevOpts*>(at(L.opts));
  D.st = inst->d_st;
  D.opts = inst->d_opts;
  D.Eloc = reinterpret_cast<double*>(at(L.eloc));
  D.Gloc = reinterpret_cast<double*>(at(L.gloc));
  D.partials = reinterpret_cast<double*>(at(L.partials));
  // keep only what later calls need on the host
  hp.rest64.clear(); hp.rest64.shrink_to_fit();
  hp.rest32.clear(); hp.rest32.shrink_to_fit();
  hp.tile_nodes.clear(); hp.tile_nodes.shrink_to_fit();
  hp.tet_loc.clear(); hp.tet_loc.shrink_to_fit();
  hp.seg_c.clear(); hp.seg_c.shrink_to_fit();
  hp.nseg_c.clear(); hp.nseg_c.shrink_to_fit();
  hp.slot_col.clear(); hp.slot_col.shrink_to_fit();
  return PHX_OK;
}

// Makes the context's pinned staging hold `bytes`, once the last copy from it is done.
// Returns false if pinned memory cannot be had (the caller then stages in pageable memory).
bool stage_reserve(phx_context ctx, size_t bytes) {
  if (ctx->stage_ev && cudaEventSynchronize(ctx->stage_ev) != cudaSuccess) return false;
  if (bytes <= ctx->stage_cap) return true;
  if (ctx->stage) cudaFreeHost(ctx->stage);
  ctx->stage = nullptr;
  ctx->stage_cap = 0;
  const size_t cap = (bytes + ((size_t)1 << 20) - 1) & ~(((size_t)1 << 20) - 1);
  if (cudaMallocHost(&ctx->stage, cap) != cudaSuccess) {
    cudaGetLastError();
    ctx->stage = nullptr;
    return false;
  }
  ctx->stage_cap = cap;
  return true;
}
int stage_done(phx_context ctx) {  // after the copies from the staging buffer are queued
  if (!ctx->stage_ev) CU(cudaEventCreateWithFlags(&ctx->stage_ev, cudaEventDisableTiming));
  CU(cudaEventRecord(ctx->stage_ev, ctx->stream));
  return PHX_OK;
}

// One instance's device part from its host pattern and rest positions (single set-ups: the
// server's admissions and rebuilds, which must not wait for the kernels running on the stream).
// The packed upload is pageable: the runtime copies it into its own staging before the call
// returns, so the buffer may be released at once and nothing waits for the stream.
int instance_setup_device(phx_context ctx, const phx_mesh* mesh, phx_instance_s* inst, bool keep_on_fail = false) {
  const BaseLayout L = base_layout(inst->hp);
  std::vector<char> buf;
  try {
    buf.resize(L.upload_end);
  } catch (const std::bad_alloc&) {
    if (keep_on_fail) instance_free_device(inst);
    else phx_instance_destroy(inst);
    return set_err(PHX_ENOMEM, "out of host memory staging an instance");
  }
  pack_base(inst->hp, mesh->X0, L, buf.data());
  return setup_from_stage(ctx, inst, L, buf.data(), keep_on_fail);
}

}  // namespace

int phx_instance_create(phx_context ctx, const phx_mesh* mesh, phx_instance* out) {
  return phx_instances_create(ctx, 1, mesh, out);
}

// Builds the host parts of count instances on up to hardware_concurrency() threads, then
// sets them up on the device one after the other with one synchronisation at the end.
int phx_instances_create(phx_context ctx, int32_t count, const phx_mesh* meshes, phx_instance* out) {
  if (!ctx || (count > 0 && (!meshes || !out)) || count < 0) return set_err(PHX_EINVAL, "NULL argument");
  for (int32_t i = 0; i < count; ++i) out[i] = nullptr;
  if (count == 0) return PHX_OK;
  std::vector<phx_instance_s*> insts;
  std::vector<std::string> errs;
  std::vector<char> ok;
  try {  // no exception may cross the C ABI: a refused host allocation is PHX_ENOMEM
    insts.assign(count, nullptr);
    errs.resize(count);
    ok.assign(count, 0);
    for (int32_t i = 0; i < count; ++i) {
      insts[i] = new phx_instance_s();
      insts[i]->ctx = ctx;
    }
  } catch (const std::bad_alloc&) {
    for (auto* p : insts) delete p;
    return set_err(PHX_ENOMEM, "out of host memory creating instances");
  }
  std::atomic<int32_t> next{0};
  auto work = [&]() {  // nothing may leave a worker thread (or cross the C ABI) as an exception
    for (int32_t i; (i = next.fetch_add(1)) < count;) {
      try {
        ok[i] = instance_build_host(&meshes[i], insts[i], errs[i]);
      } catch (const std::bad_alloc&) {
        errs[i] = "out of host memory building the pattern";
      } catch (...) {
        errs[i] = "unexpected error building the pattern";
      }
    }
  };
  const int nt = std::max(1, std::min<int>(count, (int)std::thread::hardware_concurrency()));
  {
    // the calling thread works too; if the system refuses a thread, the ones started share
    // the work (a thread left unjoined would end the process)
    std::vector<std::thread> pool;
    try {
      for (int t = 1; t < nt; ++t) pool.emplace_back(work);
    } catch (const std::system_error&) {
    }
    work();
    for (auto& th : pool) th.join();
  }
  for (int32_t i = 0; i < count; ++i)
    if (!ok[i]) {
      for (auto* p : insts) delete p;
      const int code = errs[i].rfind("out of host memory", 0) == 0 ? PHX_ENOMEM : PHX_EINVAL;
      return set_err(code, count == 1 ? errs[i] : "mesh " + std::to_string(i) + ": " + errs[i]);
    }
  cudaError_t e = cudaSetDevice(ctx->device);
  if (e != cudaSuccess) {
    for (auto* p : insts) delete p;
    return set_err(PHX_ECUDA, cudaGetErrorString(e));
  }
  // every instance's upload packed into one pinned staging buffer (on the host threads), then
  // one arena block, one copy and one memset per instance
  std::vector<BaseLayout> lay(count);
  std::vector<size_t> at(count + 1, 0);
  for (int32_t i = 0; i < count; ++i) {
    lay[i] = base_layout(insts[i]->hp);
    at[i + 1] = at[i] + ((lay[i].upload_end + 255) & ~(size_t)255);
  }
  const bool staged = stage_reserve(ctx, at[count]);
  if (staged) {
    std::atomic<int32_t> nxt{0};
    auto pack = [&]() {
      for (int32_t i; (i = nxt.fetch_add(1)) < count;) pack_base(insts[i]->hp, meshes[i].X0, lay[i], ctx->stage + at[i]);
    };
    std::vector<std::thread> pool;
    try {
      for (int t = 1; t < nt; ++t) pool.emplace_back(pack);
    } catch (const std::system_error&) {
    }
    pack();
    for (auto& th : pool) th.join();
  }
  for (int32_t i = 0; i < count; ++i) {
    // destroys insts[i] on failure
    const int rc = staged ? setup_from_stage(ctx, insts[i], lay[i], ctx->stage + at[i], false)
                          : instance_setup_device(ctx, &meshes[i], insts[i]);
    if (rc != PHX_OK) {
      for (int32_t j = 0; j < i; ++j) phx_instance_destroy(insts[j]);
      for (int32_t j = i + 1; j < count; ++j) delete insts[j];
      if (staged) stage_done(ctx);
      return rc;
    }
  }
  if (staged) TRY(stage_done(ctx));
  e = cudaStreamSynchronize(ctx->stream);
  if (e != cudaSuccess) {
    for (auto* p : insts) phx_instance_destroy(p);
    return set_err(PHX_ECUDA, cudaGetErrorString(e));
  }
  for (int32_t i = 0; i < count; ++i) out[i] = insts[i];
  return PHX_OK;
}

int phx_instance_sizes(phx_instance inst, int64_t* ndof, int64_t* nnz, int64_t* nlo, int64_t* nfull) {
  if (!inst) return set_err(PHX_EINVAL, "inst is NULL");
  if (inst->host_state.load(std::memory_order_acquire) != HOST_READY && !inst->resident)
    return set_err(PHX_EBUSY, "instance's pattern is not built yet");
  const HostPattern& hp = inst->hp;
  if (ndof) *ndof = 3 * (int64_t)hp.n;
  if (nnz) *nnz = 9 * (int64_t)hp.nlo;
  if (nlo) *nlo = hp.nlo;
  if (nfull) *nfull = 2 * (int64_t)hp.nlo - hp.n;
  return PHX_OK;
}

int phx_instance_reset(phx_instance inst) {
  if (!inst) return set_err(PHX_EINVAL, "inst is NULL");
  if (inst->in_server) return set_err(PHX_EBUSY, "instance is admitted to a server");
  TRY(require_resident(inst));
  const size_t bytes = 4 * (size_t)inst->dev.n * sizeof(double);
  cudaStream_t st = inst->ctx->stream;
  CU(cudaMemcpyAsync(inst->dev.x, inst->dev.xrest, bytes, cudaMemcpyDeviceToDevice, st));
  CU(cudaMemsetAsync(inst->dev.v, 0, bytes, st));
  CU(cudaMemsetAsync(inst->dev.dxprev, 0, bytes, st));
  // staged boundary conditions back to stage 0 (Simulable::ResetBoundaryConditions)
  inst->stage = 0;
  if (!inst->soft0.empty())
    CU(cudaMemcpyAsync(inst->dev.soft, inst->soft0.data(), inst->soft0.size() * sizeof(double),
                       cudaMemcpyHostToDevice, st));
  return PHX_OK;
}

}  // extern "C"

namespace {

// Frees the device copies of an instance's staging arrays (the host copies stay).
int release_staging(phx_instance inst) {
  int64_t freed = 0;
  InstDev& D = inst->dev;
  CU(cudaStreamSynchronize(inst->ctx->stream));
  for (const void* p : {(const void*)D.stage_grp, (const void*)D.stage_ini, (const void*)D.stage_par}) {
    if (!p) continue;
    auto it = std::find(inst->blocks.begin(), inst->blocks.end(), p);
    if (it == inst->blocks.end()) continue;
    const int64_t b = (int64_t)inst->ctx->arena.size_of(p);
    inst->ctx->arena.free(*it);
    inst->blocks.erase(it);
    inst->bytes -= b;
    freed += b;
  }
  if (inst->owner) server_account(inst->owner, -freed);
  D.stage_grp = nullptr;
  D.stage_ini = nullptr;
  D.stage_par = nullptr;
  return PHX_OK;
}

// Uploads the instance's staging arrays and its stage-0 soft records; `account`: the bytes
// count against the instance's server at once (a server that sets an instance up counts them
// itself).
int upload_staging(phx_instance inst, bool account = true) {
  if (inst->stage_grp.empty()) return PHX_OK;
  InstDev& D = inst->dev;
  const int64_t b0 = inst->bytes;
  int32_t* dg = nullptr;
  double* di = nullptr;
  double* dp = nullptr;
  TRY(upload(inst, &dg, inst->stage_grp));
  TRY(upload(inst, &di, inst->stage_ini));
  TRY(upload(inst, &dp, inst->stage_par));
  D.stage_grp = dg;
  D.stage_ini = di;
  D.stage_par = dp;
  if (inst->owner && account) server_account(inst->owner, inst->bytes - b0);
  if (!inst->soft0.empty() && D.soft)
    CU(cudaMemcpyAsync(D.soft, inst->soft0.data(), inst->soft0.size() * sizeof(double), cudaMemcpyHostToDevice,
                       inst->ctx->stream));
  CU(cudaStreamSynchronize(inst->ctx->stream));
  return PHX_OK;
}

}  // namespace

extern "C" {

// Staged boundary conditions: BCondition stages (BCondition.cpp:42-67) over groups of
// BC_FixDoF nodes with VectorAnimator_LerpT3D targets (BC_FixDoF.cpp:80-121).
int phx_instance_set_staging(phx_instance inst, int32_t count, const phx_stage_group* groups, int32_t num_stages) {
  if (!inst || count < 0 || num_stages < 0 || (count > 0 && !groups)) return set_err(PHX_EINVAL, "bad arguments");
  if (inst->in_server) return set_err(PHX_EBUSY, "instance is admitted to a server");
  TRY(require_resident(inst));
  if (count > 64) return set_err(PHX_EINVAL, "staging: at most 64 groups");
  const HostPattern& hp = inst->hp;
  const int n = hp.n;
  std::vector<int32_t> grp(n, -1);
  std::vector<double> par(16 * (size_t)std::max(count, 1), 0.0);
  int most = num_stages;
  bool values = false;
  for (int g = 0; g < count; ++g) {
    const phx_stage_group& G = groups[g];
    if (G.num_stages < 1 || G.num_nodes < 0 || (G.num_nodes > 0 && !G.nodes))
      return set_err(PHX_EINVAL, "staging: group " + std::to_string(g) + " needs num_stages >= 1 and its nodes");
    for (int k = 0; k < G.num_nodes; ++k) {
      const int v = G.nodes[k];
      if (v < 0 || v >= n) return set_err(PHX_EINVAL, "staging: node id out of range");
      if (grp[v] >= 0) return set_err(PHX_EINVAL, "staging: node " + std::to_string(v) + " in two groups");
      if (G.soft) {
        if (hp.soft.empty() || hp.soft[4 * (size_t)v + 3] == 0.0)
          return set_err(PHX_EINVAL, "staging: soft group node " + std::to_string(v) + " has no soft record");
      } else if ((hp.fixmask[v] & 7) != 7) {
        return set_err(PHX_EINVAL, "staging: hard group node " + std::to_string(v) + " is not fixed");
      }
      grp[v] = g;
    }
    double* P = &par[16 * (size_t)g];
    P[0] = G.num_stages;
    P[1] = G.soft ? 1.0 : 0.0;
    P[2] = G.k_start;
    P[3] = G.k_end;
    for (int k = 0; k < 9; ++k) P[4 + k] = G.move[k];
    for (int k = 0; k < 3; ++k) P[13 + k] = G.shift[k];
    bool moves = false;
    for (int k = 0; k < 12; ++k) moves = moves || P[4 + k] != 0.0;
    values = values || G.soft || moves;
    most = std::max(most, G.num_stages);
  }
  // start values: the nodes' positions now (BC_FixDoF holds the DoFs' values when it is made)
  std::vector<double> x(3 * (size_t)n), ini(4 * (size_t)n, 0.0);
  TRY(download_x(inst, inst->dev.x, x.data()));
  for (int v = 0; v < n; ++v)
    if (grp[v] >= 0)
      for (int c = 0; c < 3; ++c) ini[4 * (size_t)v + c] = x[3 * (size_t)v + c];
  TRY(release_staging(inst));
  inst->num_stages = most;
  inst->stage = 0;
  inst->stage_values = values;
  inst->soft0.clear();
  if (count == 0) return PHX_OK;
  inst->stage_grp = std::move(grp);
  inst->stage_ini = std::move(ini);
  inst->stage_par = std::move(par);
  // stage 0 of the soft groups: targets at their start values, stiffness k_start
  if (!hp.soft.empty()) {
    inst->soft0 = hp.soft;
    for (int v = 0; v < n; ++v)
      if (inst->stage_grp[v] >= 0 && groups[inst->stage_grp[v]].soft) {
        for (int c = 0; c < 3; ++c) inst->soft0[4 * (size_t)v + c] = inst->stage_ini[4 * (size_t)v + c];
        inst->soft0[4 * (size_t)v + 3] = groups[inst->stage_grp[v]].k_start;
      }
  }
  return upload_staging(inst);
}

int phx_instance_stage(phx_instance inst, int32_t* stage, int32_t* num_stages) {
  if (!inst) return set_err(PHX_EINVAL, "inst is NULL");
  if (stage) *stage = inst->stage;
  if (num_stages) *num_stages = inst->num_stages;
  return PHX_OK;
}

int phx_instance_set_positions(phx_instance inst, const double* x) {
  if (!inst || !x) return set_err(PHX_EINVAL, "NULL argument");
  TRY(require_resident(inst));
  return upload_x(inst, x, inst->dev.x);
}
// An instance off the device reports the state its server kept on the host (its rest
// shape and zero velocity if it was never admitted).
int phx_instance_get_positions(phx_instance inst, double* x) {
  if (!inst || !x) return set_err(PHX_EINVAL, "NULL argument");
  if (!inst->resident) {
    if (!inst->saved_x.empty()) std::copy(inst->saved_x.begin(), inst->saved_x.end(), x);
    else if (inst->kept) std::copy(inst->kept->X0.begin(), inst->kept->X0.end(), x);
    else return require_resident(inst);
    return PHX_OK;
  }
  return download_x(inst, inst->dev.x, x);
}
int phx_instance_set_velocities(phx_instance inst, const double* v) {
  if (!inst || !v) return set_err(PHX_EINVAL, "NULL argument");
  TRY(require_resident(inst));
  return upload_x(inst, v, inst->dev.v);
}
int phx_instance_get_velocities(phx_instance inst, double* v) {
  if (!inst || !v) return set_err(PHX_EINVAL, "NULL argument");
  if (!inst->resident) {
    if (!inst->saved_v.empty()) std::copy(inst->saved_v.begin(), inst->saved_v.end(), v);
    else if (inst->kept) std::fill(v, v + 3 * (size_t)inst->kept->n, 0.0);
    else return require_resident(inst);
    return PHX_OK;
  }
  return download_x(inst, inst->dev.v, v);
}

int phx_instance_update_load(phx_instance inst, const double* force, const double* gravity) {
  if (!inst) return set_err(PHX_EINVAL, "inst is NULL");
  if (inst->in_server) return set_err(PHX_EBUSY, "instance is admitted to a server");
  HostPattern& hp = inst->hp;
  if (inst->kept) {  // a server instance is (re)built from its kept mesh: keep its loads there too
    if (force) inst->kept->force.assign(force, force + 3 * (size_t)inst->kept->n);
    if (gravity) for (int c = 0; c < 3; ++c) inst->kept->gravity[c] = gravity[c];
  }
  if (!inst->resident) {  // applied when the server builds the instance again
    if (force) inst->force.assign(force, force + 3 * (size_t)inst->kept->n);
    if (gravity) for (int c = 0; c < 3; ++c) inst->gravity[c] = gravity[c];
    return PHX_OK;
  }
  if (force) inst->force.assign(force, force + 3 * (size_t)hp.n);
  if (gravity) for (int c = 0; c < 3; ++c) inst->gravity[c] = gravity[c];
  MeshIn in;
  in.n = hp.n;
  in.force = inst->force.empty() ? nullptr : inst->force.data();
  for (int c = 0; c < 3; ++c) in.gravity[c] = inst->gravity[c];
  rebuild_load(in, hp);
  CU(cudaMemcpyAsync(inst->dev.hlin, hp.hlin.data(), hp.hlin.size() * sizeof(double), cudaMemcpyHostToDevice,
                     inst->ctx->stream));
  CU(cudaStreamSynchronize(inst->ctx->stream));
  return PHX_OK;
}

int phx_solve_log(phx_instance inst, double* obj, double* opt, int32_t* bis, double* step, int32_t cap) {
  if (!inst) return set_err(PHX_EINVAL, "inst is NULL");
  TRY(require_resident(inst));
  NState s;
  TRY(read_state(inst, &s));
  std::vector<double> lg(4 * (size_t)kLogCap);
  CU(cudaMemcpy(lg.data(), inst->dev.log, lg.size() * sizeof(double), cudaMemcpyDeviceToHost));
  int n = std::min(std::min(s.log_count, kLogCap), std::max(cap, 0));
  for (int i = 0; i < n; ++i) {
    if (obj) obj[i] = lg[4 * i];
    if (opt) opt[i] = lg[4 * i + 1];
    if (bis) bis[i] = (int32_t)lg[4 * i + 2];
    if (step) step[i] = lg[4 * i + 3];
  }
  return s.log_count;
}

int phx_hessian_pattern(phx_instance inst, int32_t* colptr, int32_t* rowidx) {
  if (!inst || !colptr || !rowidx) return set_err(PHX_EINVAL, "NULL argument");
  if (inst->host_state.load(std::memory_order_acquire) != HOST_READY && !inst->resident)
    return set_err(PHX_EBUSY, "instance's pattern is not built yet");
  const HostPattern& hp = inst->hp;
  int64_t q = 0;
  for (int C = 0; C < hp.n; ++C)
    for (int b = 0; b < 3; ++b) {
      colptr[3 * C + b] = (int32_t)q;
      for (int k = hp.lo_colptr[C]; k < hp.lo_colptr[C + 1]; ++k) {
        int R = hp.lo_rc[2 * (size_t)k];
        for (int a = 0; a < 3; ++a) rowidx[q++] = 3 * R + a;
      }
    }
  colptr[3 * hp.n] = (int32_t)q;
  return PHX_OK;
}

int phx_scatter_map(phx_instance inst, int32_t* map) {
  if (!inst || !map) return set_err(PHX_EINVAL, "NULL argument");
  if (inst->host_state.load(std::memory_order_acquire) != HOST_READY && !inst->resident)
    return set_err(PHX_EBUSY, "instance's pattern is not built yet");
  std::copy(inst->hp.scatter.begin(), inst->hp.scatter.end(), map);
  return PHX_OK;
}

}  // extern "C"

namespace {

// Runs only the given kernels for one instance whose state is set to `phase`.
int run_kernels(phx_instance inst, const std::vector<KernelId>& ids, bool fp64) {
  phx_context ctx = inst->ctx;
  BatchDev B{};
  Grids G;
  TRY(set_batch(ctx, {inst}, B, G));
  for (KernelId id : ids) {
    int grid = 1;
    switch (id) {
      case K_ELEM_EG: case K_ELEM_HESS: grid = G.tet; break;
      case K_ASSEMBLE: grid = G.lob; break;
      default: grid = G.node; break;
    }
    do_launch(ctx, id, grid, B, fp64);
  }
  CU(cudaGetLastError());
  CU(cudaStreamSynchronize(ctx->stream));
  return PHX_OK;
}

int eval_eg(phx_instance inst, const double* x, int nofix, NState* s) {
  if (x) TRY(upload_x(inst, x, inst->dev.x));
  DevOpts d{};
  d.precision = 0;
  CU(cudaMemcpyAsync(inst->d_opts, &d, sizeof(DevOpts), cudaMemcpyHostToDevice, inst->ctx->stream));
  TRY(reset_state(inst, PH_EVAL, nofix, 0.0));
  TRY(run_kernels(inst, {K_ELEM_EG, K_GATHER}, true));
  return read_state(inst, s);
}

int eval_hess(phx_instance inst, const double* x, bool fp64, int nofix) {
  if (x) TRY(upload_x(inst, x, inst->dev.x));
  TRY(ensure_precision(inst, fp64));
  DevOpts d{};
  d.precision = fp64 ? 0 : 1;
  d.precond = 1;
  CU(cudaMemcpyAsync(inst->d_opts, &d, sizeof(DevOpts), cudaMemcpyHostToDevice, inst->ctx->stream));
  TRY(reset_state(inst, PH_HESS, nofix, 0.0));
  return run_kernels(inst, {K_ELEM_HESS, K_ASSEMBLE}, fp64);
}

}  // namespace

extern "C" {

int phx_energy_gradient(phx_instance inst, const double* x, double* energy, double* gradient, int32_t fix) {
  if (!inst) return set_err(PHX_EINVAL, "inst is NULL");
  TRY(require_resident(inst));
  NState s;
  TRY(eval_eg(inst, x, fix ? 0 : 1, &s));
  if (energy) *energy = s.E_eval;
  if (gradient) TRY(download_x(inst, inst->dev.gn, gradient));
  return PHX_OK;
}

int phx_hessian(phx_instance inst, const double* x, int32_t precision, double* values, int32_t fix) {
  if (!inst || !values) return set_err(PHX_EINVAL, "NULL argument");
  if (precision != PHX_PREC_FP64 && precision != PHX_PREC_FP32_REFINE) return set_err(PHX_EINVAL, "precision");
  TRY(require_resident(inst));
  const bool fp64 = precision == PHX_PREC_FP64;
  TRY(eval_hess(inst, x, fp64, fix ? 0 : 1));
  const HostPattern& hp = inst->hp;
  const size_t nv = 9 * (size_t)hp.nslots;
  std::vector<double> H(nv);
  if (fp64) {
    CU(cudaMemcpy(H.data(), inst->dev.H64, nv * sizeof(double), cudaMemcpyDeviceToHost));
  } else {
    std::vector<float> Hf(nv);
    CU(cudaMemcpy(Hf.data(), inst->dev.H32, nv * sizeof(float), cudaMemcpyDeviceToHost));
    for (size_t k = 0; k < nv; ++k) H[k] = Hf[k];
  }
  // CSC position of lower block k entry (a, b): column 3C+b starts at 9*lo_colptr[C] + 3*b*len(C)
  for (int C = 0; C < hp.n; ++C) {
    const int k0 = hp.lo_colptr[C], len = hp.lo_colptr[C + 1] - k0;
    for (int k = k0; k < k0 + len; ++k)
      for (int a = 0; a < 3; ++a)
        for (int b = 0; b < 3; ++b) {
          size_t pos = 9 * (size_t)k0 + 3 * (size_t)b * len + 3 * (size_t)(k - k0) + a;
          values[pos] = H[sell_addr(hp.lo_slot[k], a * 3 + b)];
        }
  }
  return PHX_OK;
}

int phx_element_local(phx_instance inst, const double* x, int32_t precision, double* E, double* g, double* Hout) {
  if (!inst) return set_err(PHX_EINVAL, "inst is NULL");
  if (precision != PHX_PREC_FP64 && precision != PHX_PREC_FP32_REFINE) return set_err(PHX_EINVAL, "precision");
  TRY(require_resident(inst));
  const int m = inst->dev.m;
  const bool fp64 = precision == PHX_PREC_FP64;
  NState s;
  TRY(eval_eg(inst, x, 0, &s));
  if (E) CU(cudaMemcpy(E, inst->dev.Eloc, m * sizeof(double), cudaMemcpyDeviceToHost));
  if (g) CU(cudaMemcpy(g, inst->dev.Gloc, 12 * (size_t)m * sizeof(double), cudaMemcpyDeviceToHost));
  if (Hout) {
    TRY(eval_hess(inst, nullptr, fp64, 0));
    std::vector<double> Hl(90 * (size_t)m);
    if (fp64) {
      CU(cudaMemcpy(Hl.data(), inst->dev.Hloc64, Hl.size() * sizeof(double), cudaMemcpyDeviceToHost));
    } else {
      std::vector<float> Hf(Hl.size());
      CU(cudaMemcpy(Hf.data(), inst->dev.Hloc32, Hf.size() * sizeof(float), cudaMemcpyDeviceToHost));
      for (size_t k = 0; k < Hf.size(); ++k) Hl[k] = Hf[k];
    }
    const int32_t* T = inst->hp.tets.data();
    for (int e = 0; e < m; ++e) {
      double* He = Hout + 144 * (size_t)e;
      for (int p = 0; p < 10; ++p) {
        int li = kPairI[p], lj = kPairJ[p];
        bool keep = T[4 * (size_t)e + li] >= T[4 * (size_t)e + lj];  // block stored as (li, lj)
        const double* blk = &Hl[90 * (size_t)e + 9 * p];
        for (int a = 0; a < 3; ++a)
          for (int b = 0; b < 3; ++b) {
            double v = blk[a * 3 + b];
            int r = keep ? 3 * li + a : 3 * lj + a;
            int c = keep ? 3 * lj + b : 3 * li + b;
            He[r * 12 + c] = v;
            He[c * 12 + r] = v;
          }
      }
    }
  }
  return PHX_OK;
}

int phx_instance_sample_grid(phx_instance inst, const double* x, int32_t field, const phx_grid* grid, double fill,
                             double* values, int32_t* owner) {
  if (!inst || !grid || !values) return set_err(PHX_EINVAL, "NULL argument");
  if (field < PHX_FIELD_DISPLACEMENT_X || field > PHX_FIELD_ENERGY_DENSITY)
    return set_err(PHX_EINVAL, "unknown field " + std::to_string(field));
  int64_t count = 1;
  for (int d = 0; d < 3; ++d) {
    if (grid->shape[d] < 1) return set_err(PHX_EINVAL, "grid: every shape entry must be >= 1");
    if (!std::isfinite(grid->origin[d]) || !(grid->delta[d] > 0.0) || !std::isfinite(grid->delta[d]))
      return set_err(PHX_EINVAL, "grid: origin must be finite and delta positive");
    count *= grid->shape[d];
    if (count > INT32_MAX) return set_err(PHX_EINVAL, "grid: more than 2^31 - 1 values");
  }
  TRY(require_resident(inst));
  phx_context ctx = inst->ctx;
  if (field == PHX_FIELD_ENERGY_DENSITY) {
    NState s;
    TRY(eval_eg(inst, x, 0, &s));
  } else if (x) {
    TRY(upload_x(inst, x, inst->dev.x));
  }
  int32_t* d_owner = (int32_t*)ctx->arena.alloc((size_t)count * sizeof(int32_t));
  double* d_values = (double*)ctx->arena.alloc((size_t)count * sizeof(double));
  auto release = [&] {
    ctx->arena.free(d_owner);
    ctx->arena.free(d_values);
  };
  if (!d_owner || !d_values) {
    release();
    return set_err(PHX_ENOMEM, "device arena exhausted (grid of " + std::to_string(count) + " values)");
  }
  GridSampleArgs a{};
  a.n = inst->dev.n;
  a.m = inst->dev.m;
  a.tets = inst->dev.tets;
  a.xrest = inst->dev.xrest;
  a.x = inst->dev.x;
  a.energy = inst->dev.Eloc;
  a.field = field;
  for (int d = 0; d < 3; ++d) {
    a.shape[d] = grid->shape[d];
    a.origin[d] = grid->origin[d];
    a.delta[d] = grid->delta[d];
  }
  a.fill = fill;
  a.owner = d_owner;
  a.values = d_values;
  cudaError_t e = launch_grid_sample(ctx->stream, a, ctx->num_sms);
  ctx->launches += 3;
  if (e == cudaSuccess)
    e = cudaMemcpyAsync(values, d_values, (size_t)count * sizeof(double), cudaMemcpyDeviceToHost, ctx->stream);
  if (e == cudaSuccess && owner)
    e = cudaMemcpyAsync(owner, d_owner, (size_t)count * sizeof(int32_t), cudaMemcpyDeviceToHost, ctx->stream);
  cudaError_t es = cudaStreamSynchronize(ctx->stream);  // nothing of the grid's may be in flight once freed
  if (e == cudaSuccess) e = es;
  release();
  if (e != cudaSuccess) return set_err(PHX_ECUDA, cudaGetErrorString(e));
  return PHX_OK;
}

int phx_solve_static(phx_instance inst, const phx_options* o, double* x, phx_report* rep) {
  if (!inst) return set_err(PHX_EINVAL, "inst is NULL");
  if (inst->in_server) return set_err(PHX_EBUSY, "instance is admitted to a server");
  TRY(require_resident(inst));
  auto t0 = clk::now();
  if (x) TRY(upload_x(inst, x, inst->dev.x));
  TRY(start_solve(inst, o, false, 0.0, 0));
  TRY(run_to_completion(inst->ctx, {inst}, o->precision == PHX_PREC_FP64, o->pcg_chunk));
  NState s;
  TRY(read_state(inst, &s));
  if (wants_fp64_finish(o, s)) {
    std::vector<NState> second;
    TRY(finish_fp64(inst->ctx, {inst}, o, {s}, &second));
    if (x) TRY(download_x(inst, inst->dev.x, x));
    fill_report_finished(s, second[0], std::chrono::duration<double>(clk::now() - t0).count(), rep);
    return PHX_OK;
  }
  if (x) TRY(download_x(inst, inst->dev.x, x));
  fill_report(s, false, std::chrono::duration<double>(clk::now() - t0).count(), rep);
  return PHX_OK;
}

int phx_solve_step(phx_instance inst, const phx_options* o, double* x, phx_report* rep) {
  if (!inst) return set_err(PHX_EINVAL, "inst is NULL");
  if (inst->in_server) return set_err(PHX_EBUSY, "instance is admitted to a server");
  TRY(require_resident(inst));
  auto t0 = clk::now();
  if (x) TRY(upload_x(inst, x, inst->dev.x));
  TRY(start_solve(inst, o, false, 0.0, 1));
  TRY(run_to_completion(inst->ctx, {inst}, o->precision == PHX_PREC_FP64, o->pcg_chunk));
  NState s;
  TRY(read_state(inst, &s));
  if (x) TRY(download_x(inst, inst->dev.x, x));
  fill_report(s, true, std::chrono::duration<double>(clk::now() - t0).count(), rep);
  return PHX_OK;
}

int phx_dynamic_step(phx_instance inst, const phx_options* o, double dt, double* x, double* v, phx_report* rep) {
  if (!inst) return set_err(PHX_EINVAL, "inst is NULL");
  if (!(dt > 0)) return set_err(PHX_EINVAL, "dt must be positive");
  if (inst->in_server) return set_err(PHX_EBUSY, "instance is admitted to a server");
  TRY(require_resident(inst));
  auto t0 = clk::now();
  if (x) TRY(upload_x(inst, x, inst->dev.x));
  if (v) TRY(upload_x(inst, v, inst->dev.v));
  TRY(start_solve(inst, o, true, dt, 0));
  TRY(run_to_completion(inst->ctx, {inst}, o->precision == PHX_PREC_FP64, o->pcg_chunk));
  NState s;
  TRY(read_state(inst, &s));
  if (x) TRY(download_x(inst, inst->dev.x, x));
  if (v) TRY(download_x(inst, inst->dev.v, v));
  fill_report(s, false, std::chrono::duration<double>(clk::now() - t0).count(), rep);
  return PHX_OK;
}

int phx_batch_solve(phx_context ctx, int32_t count, phx_instance* insts, const phx_options* o, double* const* x,
                    phx_report* reps) {
  if (!ctx || count < 0 || (count > 0 && !insts)) return set_err(PHX_EINVAL, "bad arguments");
  auto t0 = clk::now();
  std::vector<phx_instance> list(insts, insts + count);
  for (int i = 0; i < count; ++i) {
    if (!list[i] || list[i]->ctx != ctx) return set_err(PHX_EINVAL, "instance from another context");
    if (list[i]->in_server) return set_err(PHX_EBUSY, "instance is admitted to a server");
    TRY(require_resident(list[i]));
    for (int j = 0; j < i; ++j)
      if (list[j] == list[i]) return set_err(PHX_EINVAL, "instance listed twice");
    if (x && x[i]) TRY(upload_x(list[i], x[i], list[i]->dev.x));
    TRY(start_solve(list[i], o, false, 0.0, 0));
  }
  if (count == 0) return PHX_OK;
  TRY(run_to_completion(ctx, list, o->precision == PHX_PREC_FP64, o->pcg_chunk));
  std::vector<NState> st, fin_first, fin_second;
  std::vector<phx_instance> fin;
  std::vector<int> fin_at(count, -1);
  TRY(read_batch(ctx, list, st, nullptr));
  for (int i = 0; i < count; ++i) {
    if (wants_fp64_finish(o, st[i])) {
      fin_at[i] = (int)fin.size();
      fin.push_back(list[i]);
      fin_first.push_back(st[i]);
    }
  }
  if (!fin.empty()) TRY(finish_fp64(ctx, fin, o, fin_first, &fin_second));
  if (x) {  // positions of the whole batch, one synchronisation
    std::vector<NState> after;
    TRY(read_batch(ctx, list, after, x));
  }
  double secs = std::chrono::duration<double>(clk::now() - t0).count();
  for (int i = 0; i < count; ++i) {
    if (!reps) continue;
    if (fin_at[i] >= 0) fill_report_finished(st[i], fin_second[fin_at[i]], secs, &reps[i]);
    else fill_report(st[i], false, secs, &reps[i]);
  }
  return PHX_OK;
}

int phx_context_launch_settings(phx_context ctx, phx_launch_settings* get, const phx_launch_settings* set) {
  if (!ctx) return set_err(PHX_EINVAL, "ctx is NULL");
  if (get) *get = ctx->launch;
  if (set) {
    if ((set->graph != 0 && set->graph != 1) || set->wait_rounds < 1 || set->wait_rounds > 64 ||
        set->wait_share < 1 || set->wait_share > 64 || set->rounds < 1 || set->rounds > 1024 ||
        (set->pcg_grid != 0 && set->pcg_grid != 1) || set->slice_share < 0 || set->slice_share > 64 ||
        set->slice_min < 1 || set->slice_min > 1000000)
      return set_err(PHX_EINVAL, "launch settings out of range");
    ctx->launch = *set;
  }
  return PHX_OK;
}

int phx_tune_batch(phx_context ctx, int32_t count, phx_instance* insts, const phx_options* o,
                   phx_launch_settings* chosen, double* default_seconds, double* best_seconds, int32_t* trials) {
  if (!ctx || !o || count <= 0 || !insts) return set_err(PHX_EINVAL, "bad arguments");
  std::vector<phx_instance> list(insts, insts + count);
  for (int i = 0; i < count; ++i) {
    if (!list[i] || list[i]->ctx != ctx) return set_err(PHX_EINVAL, "instance from another context");
    if (list[i]->in_server) return set_err(PHX_EBUSY, "instance is admitted to a server");
    if (list[i]->num_stages > 1) return set_err(PHX_EINVAL, "instances with staged boundary conditions are not tuned");
    TRY(require_resident(list[i]));
    for (int j = 0; j < i; ++j)
      if (list[j] == list[i]) return set_err(PHX_EINVAL, "instance listed twice");
  }
  TRY(validate_opts(o));
  const bool fp64 = o->precision == PHX_PREC_FP64;
  // every trial starts from the same positions and warm-start steps, put back at the end
  std::vector<std::vector<double>> x0(count), d0(count);
  for (int i = 0; i < count; ++i) {
    x0[i].resize(3 * (size_t)list[i]->dev.n);
    d0[i].resize(3 * (size_t)list[i]->dev.n);
    TRY(download_x(list[i], list[i]->dev.x, x0[i].data()));
    TRY(download_x(list[i], list[i]->dev.dxprev, d0[i].data()));
  }
  auto restore = [&]() -> int {
    for (int i = 0; i < count; ++i) {
      TRY(upload_x(list[i], x0[i].data(), list[i]->dev.x));
      TRY(upload_x(list[i], d0[i].data(), list[i]->dev.dxprev));
    }
    return PHX_OK;
  };
  int ntrials = 0;
  auto trial = [&](const phx_launch_settings& S, double* secs) -> int {
    TRY(restore());
    for (int i = 0; i < count; ++i) TRY(start_solve(list[i], o, false, 0.0, 0));
    CU(cudaStreamSynchronize(ctx->stream));
    const auto t = clk::now();
    TRY(run_to_completion(ctx, list, fp64, o->pcg_chunk, &S));
    CU(cudaStreamSynchronize(ctx->stream));
    *secs = std::chrono::duration<double>(clk::now() - t).count();
    ++ntrials;
    return PHX_OK;
  };
  phx_launch_settings best = ctx->launch;
  double t_def = 0.0, t = 0.0, t_best = 0.0;
  // the search; a trial that fails ends it, and the instances are put back all the same
  auto search = [&]() -> int {
    TRY(trial(best, &t_def));  // the first run pays one-time costs (graph, caches)
    TRY(trial(best, &t_def));
    t_best = t_def;
    // one setting at a time around the best so far
    auto consider = [&](phx_launch_settings c) -> int {
      TRY(trial(c, &t));
      if (t < 0.99 * t_best) {
        best = c;
        t_best = t;
      }
      return PHX_OK;
    };
    {
      phx_launch_settings c = best;
      c.graph = 1 - c.graph;
      TRY(consider(c));
    }
    bool eligible = false;  // FP32 instances above the cluster size: try the other place for their PCG
    for (auto* in : list) eligible = eligible || in->grid_eligible;
    if (eligible) {
      phx_launch_settings c = best;
      c.pcg_grid = 1 - c.pcg_grid;
      TRY(consider(c));
    }
    for (int v : {2, 8, 16}) {
      phx_launch_settings c = best;
      if (v == c.wait_rounds) continue;
      c.wait_rounds = v;
      TRY(consider(c));
    }
    for (int v : {1, 4, 8}) {
      phx_launch_settings c = best;
      if (v == c.wait_share) continue;
      c.wait_share = v;
      TRY(consider(c));
    }
    for (int v : {8, 32, 64}) {
      phx_launch_settings c = best;
      if (v == c.rounds) continue;
      c.rounds = v;
      TRY(consider(c));
    }
    for (int v : {0, 4, 8}) {  // cluster-PCG time slices: off, or once a quarter / an eighth of the clusters idle
      phx_launch_settings c = best;
      if (v == c.slice_share) continue;
      c.slice_share = v;
      TRY(consider(c));
    }
    if (best.slice_share > 0)
      for (int v : {16, 64, 128}) {
        phx_launch_settings c = best;
        if (v == c.slice_min) continue;
        c.slice_min = v;
        TRY(consider(c));
      }
    return PHX_OK;
  };
  const int rc = search();
  if (rc != PHX_OK) {
    const std::string why = phx_last_error();
    restore();
    cudaStreamSynchronize(ctx->stream);
    return set_err(rc, why);
  }
  TRY(restore());
  CU(cudaStreamSynchronize(ctx->stream));
  ctx->tuned[mix_key(list, fp64)] = best;
  if (chosen) *chosen = best;
  if (default_seconds) *default_seconds = t_def;
  if (best_seconds) *best_seconds = t_best;
  if (trials) *trials = ntrials;
  return PHX_OK;
}

int phx_batch_dynamic_step(phx_context ctx, int32_t count, phx_instance* insts, const phx_options* o, double dt,
                           phx_report* reps) {
  if (!ctx || count < 0 || (count > 0 && !insts)) return set_err(PHX_EINVAL, "bad arguments");
  if (!(dt > 0)) return set_err(PHX_EINVAL, "dt must be positive");
  auto t0 = clk::now();
  std::vector<phx_instance> list(insts, insts + count);
  for (int i = 0; i < count; ++i) {
    if (!list[i] || list[i]->ctx != ctx) return set_err(PHX_EINVAL, "instance from another context");
    if (list[i]->in_server) return set_err(PHX_EBUSY, "instance is admitted to a server");
    TRY(require_resident(list[i]));
    for (int j = 0; j < i; ++j)
      if (list[j] == list[i]) return set_err(PHX_EINVAL, "instance listed twice");
    TRY(start_solve(list[i], o, true, dt, 0));
  }
  if (count == 0) return PHX_OK;
  TRY(run_to_completion(ctx, list, o->precision == PHX_PREC_FP64, o->pcg_chunk));
  double secs = std::chrono::duration<double>(clk::now() - t0).count();
  std::vector<NState> st;
  TRY(read_batch(ctx, list, st, nullptr));
  for (int i = 0; i < count; ++i)
    if (reps) fill_report(st[i], false, secs, &reps[i]);
  return PHX_OK;
}

}  // extern "C"

// ===========================================================================
// serving: continuous batching
// ===========================================================================
struct phx_server_s {
  phx_context ctx = nullptr;
  int max_slots = 0;
  int64_t budget = 0, in_use = 0, peak = 0;  // device bytes this server holds
  int64_t evictions = 0, cold_admitted = 0, refused = 0;
  phx_options opts{};
  bool fp64 = true;
  enum Kind { REQ_STATIC = 0, REQ_STEP = 1 };
  struct Req {
    phx_instance inst;
    int64_t tag;
    clk::time_point t_submit;
    int kind;
    double dt;
    int64_t counted;  // bytes added to in_use for a caller's instance while it is active
  };
  std::deque<Req> queue;
  std::vector<Req> active;
  struct Done { int64_t tag; phx_report rep; };
  std::deque<Done> done;
  bool dirty = true;
  BatchDev B{};
  Grids G;
  int ccount = 0;
  uint64_t tick = 0;
  std::vector<phx_instance> owned;  // instances this server created for cold requests
  // host parts of cold requests (validation, pattern, scatter map) are built on workers
  std::mutex mu;
  std::condition_variable cv;
  std::deque<phx_instance> jobs;
  bool stop = false;
  std::vector<std::thread> workers;
};

void server_account(phx_server s, int64_t delta) {
  s->in_use += delta;
  s->peak = std::max(s->peak, s->in_use);
}

void server_forget(phx_server s, phx_instance inst) {
  auto it = std::find(s->owned.begin(), s->owned.end(), inst);
  if (it == s->owned.end()) return;
  if (inst->resident) s->in_use -= inst->bytes;
  s->owned.erase(it);
  inst->owner = nullptr;
}

namespace {

void server_worker(phx_server s) {
  for (;;) {
    phx_instance inst = nullptr;
    {
      std::unique_lock<std::mutex> lk(s->mu);
      s->cv.wait(lk, [&] { return s->stop || !s->jobs.empty(); });
      if (s->stop) return;
      inst = s->jobs.front();
      s->jobs.pop_front();
    }
    std::string err;
    bool ok = false;
    try {
      inst->hp = HostPattern{};
      const phx_mesh v = inst->kept->view();
      ok = instance_build_host(&v, inst, err);
    } catch (const std::bad_alloc&) {
      err = "out of host memory building the pattern";
    } catch (...) {
      err = "unexpected error building the pattern";
    }
    inst->host_err = err;
    inst->host_state.store(ok ? HOST_READY : HOST_FAILED, std::memory_order_release);
  }
}

// Queues the (re)build of a server instance's host part on the workers.
int server_build_host(phx_server s, phx_instance inst) {
  if (inst->host_state.load(std::memory_order_acquire) != HOST_NONE) return PHX_OK;
  inst->host_state.store(HOST_BUILDING, std::memory_order_release);
  try {
    if (s->workers.empty()) {
      const int nt = std::max(1, std::min(8, (int)std::thread::hardware_concurrency()));
      for (int t = 0; t < nt; ++t) s->workers.emplace_back(server_worker, s);
    }
    std::lock_guard<std::mutex> lk(s->mu);
    s->jobs.push_back(inst);
  } catch (...) {
    inst->host_state.store(HOST_NONE, std::memory_order_release);
    if (s->workers.empty()) return set_err(PHX_ENOMEM, "cannot start a host-build thread");
    return set_err(PHX_ENOMEM, "out of host memory queueing a request");
  }
  s->cv.notify_one();
  return PHX_OK;
}

// Moves an idle instance of the server off the device: its positions and velocities stay on
// the host, its arena blocks are freed and its host part is rebuilt on its next request.
int server_evict(phx_server s, phx_instance inst) {
  const size_t N = 3 * (size_t)inst->dev.n;
  inst->saved_x.resize(N);
  inst->saved_v.resize(N);
  TRY(download_x(inst, inst->dev.x, inst->saved_x.data()));
  TRY(download_x(inst, inst->dev.v, inst->saved_v.data()));
  s->in_use -= inst->bytes;
  TRY(instance_free_device(inst));
  inst->host_state.store(HOST_NONE, std::memory_order_release);
  s->evictions++;
  return PHX_OK;
}

// Puts a finished request on the done list with a failure report (no solve ran).
void server_fail(phx_server s, const phx_server_s::Req& r, int status) {
  phx_report rep{};
  rep.result = OS_FAILURE;
  rep.status = status;
  rep.seconds = std::chrono::duration<double>(clk::now() - r.t_submit).count();
  s->done.push_back({r.tag, rep});
  r.inst->in_server = false;
  s->refused++;
}

// Device part of an admitted request: the instance set up on the device if it is not, with
// the buffers of the server's arithmetic.  Returns PHX_ENOMEM (nothing kept) when the arena
// cannot hold it.
int server_allocate(phx_server s, phx_instance inst) {
  const bool fresh = !inst->resident;
  if (fresh) {
    const phx_mesh v = inst->kept->view();
    TRY(instance_setup_device(s->ctx, &v, inst, true));  // on failure the host part is intact
  }
  const int rc = ensure_precision(inst, s->fp64);
  if (rc != PHX_OK) {
    if (fresh) {  // no room for its arithmetic: leave nothing behind; the set-up released the
      instance_free_device(inst);  // pattern's host copies, so it is built again
      inst->host_state.store(HOST_NONE, std::memory_order_release);
    }
    return rc;
  }
  if (fresh) {
    TRY(upload_staging(inst, false));  // counted with the rest of the set-up by the caller
    if (!inst->saved_x.empty()) TRY(upload_x(inst, inst->saved_x.data(), inst->dev.x));
    if (!inst->saved_v.empty()) TRY(upload_x(inst, inst->saved_v.data(), inst->dev.v));
    inst->saved_x.clear();
    inst->saved_v.clear();
    s->cold_admitted++;
  }
  return PHX_OK;
}

}  // namespace

extern "C" {

int phx_server_create(phx_context ctx, int32_t max_slots, int64_t budget, const phx_options* o, phx_server* out) {
  if (!ctx || !out || max_slots < 1) return set_err(PHX_EINVAL, "bad arguments");
  TRY(validate_opts(o));
  auto* s = new (std::nothrow) phx_server_s();
  if (!s) return set_err(PHX_ENOMEM, "out of host memory");
  s->ctx = ctx;
  s->max_slots = max_slots;
  s->budget = budget > 0 ? budget : (int64_t)ctx->arena.cap;
  s->opts = *o;
  s->fp64 = o->precision == PHX_PREC_FP64;
  *out = s;
  return PHX_OK;
}

int phx_server_destroy(phx_server s) {
  if (!s) return PHX_OK;
  {
    std::lock_guard<std::mutex> lk(s->mu);
    s->stop = true;
  }
  s->cv.notify_all();
  for (auto& t : s->workers) t.join();
  for (phx_instance inst : s->jobs)  // queued builds that never ran
    inst->host_state.store(HOST_NONE, std::memory_order_release);
  cudaStreamSynchronize(s->ctx->stream);
  for (auto& r : s->active) r.inst->in_server = false;
  for (auto& r : s->queue) r.inst->in_server = false;
  for (phx_instance inst : s->owned) inst->owner = nullptr;  // the caller keeps (and destroys) them
  delete s;
  return PHX_OK;
}

namespace {

int server_enqueue(phx_server s, phx_instance inst, int64_t tag, int kind, double dt) {
  if (!s || !inst || inst->ctx != s->ctx) return set_err(PHX_EINVAL, "bad arguments");
  if (inst->in_server) return set_err(PHX_EBUSY, "instance already queued or active");
  if (inst->owner && inst->owner != s) return set_err(PHX_EINVAL, "instance belongs to another server");
  if (!inst->resident && !inst->owner) return set_err(PHX_EINVAL, "instance has no device part and no server");
  if (inst->resident && !inst->owner) {
    // a caller's instance: its bytes count while it is active
    const int64_t need = inst->bytes + (s->fp64 ? (inst->have64 ? 0 : precision_bytes(inst->dev.n, inst->dev.m,
                                                                                      inst->dev.nslots, 8))
                                                : (inst->have32 ? 0 : precision_bytes(inst->dev.n, inst->dev.m,
                                                                                      inst->dev.nslots, 4)));
    if (need > s->budget) {
      s->refused++;
      return set_err(PHX_ENOMEM, "instance larger than the server budget");
    }
  }
  if (!inst->resident) TRY(server_build_host(s, inst));
  inst->in_server = true;
  s->queue.push_back({inst, tag, clk::now(), kind, dt, 0});
  return PHX_OK;
}

}  // namespace

int phx_server_submit(phx_server s, phx_instance inst, int64_t tag) {
  return server_enqueue(s, inst, tag, phx_server_s::REQ_STATIC, 0.0);
}

int phx_server_submit_step(phx_server s, phx_instance inst, double dt, int64_t tag) {
  if (!(dt > 0)) return set_err(PHX_EINVAL, "dt must be positive");
  return server_enqueue(s, inst, tag, phx_server_s::REQ_STEP, dt);
}

int phx_server_submit_mesh(phx_server s, const phx_mesh* mesh, int64_t tag, phx_instance* out) {
  if (!s || !mesh || !out) return set_err(PHX_EINVAL, "NULL argument");
  *out = nullptr;
  if (mesh->num_nodes <= 0 || mesh->num_tets <= 0 || !mesh->X0 || !mesh->tets || !mesh->lame || !mesh->rho)
    return set_err(PHX_EINVAL, "mesh: empty or missing arrays");
  phx_instance_s* inst = nullptr;
  try {
    inst = new phx_instance_s();
    inst->ctx = s->ctx;
    inst->owner = s;
    inst->resident = false;
    inst->host_state.store(HOST_NONE, std::memory_order_relaxed);
    auto k = std::make_unique<KeptMesh>();
    const size_t n = mesh->num_nodes, m = mesh->num_tets;
    k->n = mesh->num_nodes;
    k->m = mesh->num_tets;
    k->X0.assign(mesh->X0, mesh->X0 + 3 * n);
    k->T.assign(mesh->tets, mesh->tets + 4 * m);
    k->lame.assign(mesh->lame, mesh->lame + 2 * m);
    k->rho.assign(mesh->rho, mesh->rho + m);
    if (mesh->model) k->model.assign(mesh->model, mesh->model + m);
    if (mesh->fixed) k->fixed.assign(mesh->fixed, mesh->fixed + 3 * n);
    if (mesh->force) k->force.assign(mesh->force, mesh->force + 3 * n);
    if (mesh->soft_k) k->soft_k.assign(mesh->soft_k, mesh->soft_k + n);
    if (mesh->soft_target) k->soft_target.assign(mesh->soft_target, mesh->soft_target + 3 * n);
    for (int c = 0; c < 3; ++c) k->gravity[c] = mesh->gravity[c];
    inst->kept = std::move(k);
    s->owned.push_back(inst);
  } catch (const std::bad_alloc&) {
    if (inst) {
      if (!s->owned.empty() && s->owned.back() == inst) s->owned.pop_back();
      delete inst;
    }
    return set_err(PHX_ENOMEM, "out of host memory copying the mesh");
  }
  const int rc = server_enqueue(s, inst, tag, phx_server_s::REQ_STATIC, 0.0);
  if (rc != PHX_OK) {
    s->owned.pop_back();
    delete inst;
    return rc;
  }
  *out = inst;
  return PHX_OK;
}

int phx_server_stats(phx_server s, int64_t* in_use, int64_t* peak, int64_t* resident, int64_t* evictions) {
  if (!s) return set_err(PHX_EINVAL, "server is NULL");
  if (in_use) *in_use = s->in_use;
  if (peak) *peak = s->peak;
  if (resident) {
    int64_t r = 0;
    for (phx_instance inst : s->owned) r += inst->resident ? 1 : 0;
    *resident = r;
  }
  if (evictions) *evictions = s->evictions;
  return PHX_OK;
}

int phx_server_progress(phx_server s, int32_t* active, int32_t* queued) {
  if (!s) return set_err(PHX_EINVAL, "server is NULL");
  // retire finished requests (phases from the last round of this server)
  if (!s->active.empty() && !s->dirty && s->ctx->batch_owner == s) {
    std::vector<phx_server_s::Req> keep, fin;
    std::vector<NState> fin_first, fin_second;
    auto retire = [&](phx_server_s::Req& r, const phx_report& rep) {
      s->done.push_back({r.tag, rep});
      r.inst->in_server = false;
      r.inst->last_used = ++s->tick;
      s->in_use -= r.counted;
      s->dirty = true;
    };
    for (size_t i = 0; i < s->active.size(); ++i) {
      if (s->ctx->h_flags[8 + i] == PH_DONE) {
        auto& r = s->active[i];
        NState st;
        TRY(read_state(r.inst, &st));
        if (r.kind == phx_server_s::REQ_STATIC && wants_fp64_finish(&s->opts, st)) {  // finished in FP64 below
          fin.push_back(r);
          fin_first.push_back(st);
          continue;
        }
        phx_report rep{};
        fill_report(st, false, std::chrono::duration<double>(clk::now() - r.t_submit).count(), &rep);
        retire(r, rep);
      } else {
        keep.push_back(s->active[i]);
      }
    }
    s->active.swap(keep);
    if (!fin.empty()) {
      std::vector<phx_instance> insts;
      std::vector<int64_t> before;
      for (auto& r : fin) {
        insts.push_back(r.inst);
        before.push_back(r.inst->bytes);
      }
      TRY(finish_fp64(s->ctx, insts, &s->opts, fin_first, &fin_second));
      for (size_t k = 0; k < fin.size(); ++k) {
        if (fin[k].inst->owner == s) s->in_use += fin[k].inst->bytes - before[k];  // its FP64 buffers
        phx_report rep{};
        fill_report_finished(fin_first[k], fin_second[k],
                             std::chrono::duration<double>(clk::now() - fin[k].t_submit).count(), &rep);
        retire(fin[k], rep);
      }
      s->dirty = true;  // the FP64 finish used the context's batch buffers
    }
  }
  // admit queued requests at this Newton-round boundary: by slots, then by the memory
  // budget (evicting idle instances, least recently used first), in arrival order; a
  // request whose host part is still being built lets the ones behind it go first, one
  // that waits for memory holds them (large requests are not starved)
  std::deque<phx_server_s::Req> still;
  bool blocked = false;
  while (!s->queue.empty()) {
    phx_server_s::Req r = s->queue.front();
    s->queue.pop_front();
    if (blocked || (int)s->active.size() >= s->max_slots) {
      still.push_back(r);
      continue;
    }
    phx_instance inst = r.inst;
    const int hs = inst->host_state.load(std::memory_order_acquire);
    if (!inst->resident && hs == HOST_FAILED) {
      set_err(PHX_EINVAL, inst->host_err);
      server_fail(s, r, PHX_EINVAL);
      continue;
    }
    if (!inst->resident && hs != HOST_READY) {
      if (hs == HOST_NONE) TRY(server_build_host(s, inst));  // released by a failed admission
      still.push_back(r);
      continue;
    }
    const bool owned = inst->owner == s;
    const size_t es = s->fp64 ? 8 : 4;
    const bool have = s->fp64 ? inst->have64 : inst->have32;
    int64_t need;
    if (!inst->resident) {
      need = device_bytes(inst->hp, !s->fp64, s->fp64);
      if (!inst->stage_grp.empty())
        need += arena_bytes_of(inst->stage_grp.size(), 4) + arena_bytes_of(inst->stage_ini.size(), 8) +
                arena_bytes_of(inst->stage_par.size(), 8);
    }
    else need = (owned ? 0 : inst->bytes) + (have ? 0 : precision_bytes(inst->dev.n, inst->dev.m, inst->dev.nslots, es));
    std::vector<Resident> res;
    std::vector<phx_instance> cand;
    for (phx_instance o : s->owned)
      if (o != inst && o->resident) {
        res.push_back({o->bytes, o->last_used, !o->in_server});
        cand.push_back(o);
      }
    std::vector<int> plan;
    const int verdict = admit_decision((int)s->active.size(), s->max_slots, s->in_use, s->budget, need, res, &plan);
    if (verdict == NEVER) {
      set_err(PHX_ENOMEM, "instance larger than the server budget");
      server_fail(s, r, PHX_ENOMEM);
      continue;
    }
    if (verdict == WAIT_SLOTS || verdict == WAIT_MEMORY) {
      blocked = true;
      still.push_back(r);
      continue;
    }
    for (int k : plan) TRY(server_evict(s, cand[k]));
    const int64_t b0 = inst->bytes;
    int rc = server_allocate(s, inst);
    if (rc == PHX_ENOMEM) {
      // the arena itself is short (fragmentation, or memory outside this server's budget):
      // evict the remaining idle instances, least recently used first, and try once more
      std::vector<int> idle;
      for (int k = 0; k < (int)cand.size(); ++k)
        if (cand[k]->resident && !cand[k]->in_server) idle.push_back(k);
      std::stable_sort(idle.begin(), idle.end(), [&](int a, int b) { return res[a].last_used < res[b].last_used; });
      for (int k : idle) TRY(server_evict(s, cand[k]));
      if (!idle.empty()) rc = server_allocate(s, inst);
    }
    if (rc == PHX_ENOMEM) {
      blocked = true;
      still.push_back(r);
      continue;
    }
    TRY(rc);
    if (owned) {
      s->in_use += inst->bytes - b0;  // resident from now on, idle or not
    } else {
      r.counted = inst->bytes;        // a caller's instance counts while it is active
      s->in_use += r.counted;
    }
    s->peak = std::max(s->peak, s->in_use);
    TRY(start_solve(inst, &s->opts, r.kind == phx_server_s::REQ_STEP, r.dt, 0));
    inst->last_used = ++s->tick;
    s->active.push_back(r);
    s->dirty = true;
  }
  s->queue.swap(still);
  if (!s->active.empty()) {
    if (s->dirty || s->ctx->batch_owner != s) {
      std::vector<phx_instance> list;
      for (auto& r : s->active) list.push_back(r.inst);
      apply_pcg_grid(list, s->ctx->launch);
      TRY(set_batch(s->ctx, list, s->B, s->G));
      TRY(set_cluster_list(s->ctx, list, &s->ccount));
      s->ctx->batch_owner = s;
      s->dirty = false;
    }
    TRY(run_step(s->ctx, s->B, (int)s->active.size(), s->fp64, s->opts.pcg_chunk, s->ccount, s->ctx->launch));
  }
  if (active) *active = (int32_t)s->active.size();
  if (queued) *queued = (int32_t)s->queue.size();
  return PHX_OK;
}

int phx_server_poll(phx_server s, int64_t* tags, phx_report* reps, int32_t cap) {
  if (!s) return set_err(PHX_EINVAL, "server is NULL");
  int n = 0;
  while (n < cap && !s->done.empty()) {
    if (tags) tags[n] = s->done.front().tag;
    if (reps) reps[n] = s->done.front().rep;
    s->done.pop_front();
    ++n;
  }
  return n;
}

// ---- profiling -------------------------------------------------------------
int phx_profile_enable(phx_context ctx, int32_t on) {
  if (!ctx) return set_err(PHX_EINVAL, "ctx is NULL");
  if (on && !ctx->d_algo) {
    CU(cudaMalloc(&ctx->d_algo, sizeof(double) * K_COUNT));
    CU(cudaMemsetAsync(ctx->d_algo, 0, sizeof(double) * K_COUNT, ctx->stream));
  }
  ctx->profiling = on != 0;
  ctx->batch_owner = nullptr;  // batches pick the new setting up on their next round
  return PHX_OK;
}

int phx_profile_bytes(phx_context ctx, const char* kind, double* bytes) {
  if (!ctx || !kind || !bytes) return set_err(PHX_EINVAL, "bad arguments");
  *bytes = 0.0;
  if (!ctx->d_algo) return PHX_OK;
  double h[K_COUNT];
  CU(cudaMemcpyAsync(h, ctx->d_algo, sizeof(h), cudaMemcpyDeviceToHost, ctx->stream));
  CU(cudaStreamSynchronize(ctx->stream));
  for (int k = 0; k < K_COUNT; ++k)
    if (std::strcmp(kernel_name((KernelId)k), kind) == 0) {
      *bytes = h[k];
      return PHX_OK;
    }
  return set_err(PHX_ENOTFOUND, std::string("unknown kernel kind ") + kind);
}

static int collect_events(phx_context ctx) {
  CU(cudaStreamSynchronize(ctx->stream));
  if (ctx->d_stage) {
    unsigned long long h[32];
    CU(cudaMemcpy(h, ctx->d_stage, sizeof(h), cudaMemcpyDeviceToHost));
    for (int k = 0; k < K_COUNT; ++k) {
      ctx->prof_ms[k] += h[k] * 1e-6;
      ctx->prof_n[k] += (int64_t)h[16 + k];
    }
    CU(cudaMemset(ctx->d_stage, 0, sizeof(h)));
  }
  for (auto& ev : ctx->evs) {
    float ms = 0;
    CU(cudaEventElapsedTime(&ms, ev.a, ev.b));
    ctx->prof_ms[ev.kind] += ms;
    ctx->prof_n[ev.kind]++;
    ctx->pool.push_back(ev.a);
    ctx->pool.push_back(ev.b);
  }
  ctx->evs.clear();
  return PHX_OK;
}

int phx_profile_read(phx_context ctx, const char* kind, int64_t* launches, double* total_ms) {
  if (!ctx || !kind) return set_err(PHX_EINVAL, "bad arguments");
  TRY(collect_events(ctx));
  for (int k = 0; k < K_COUNT; ++k)
    if (std::strcmp(kernel_name((KernelId)k), kind) == 0) {
      if (launches) *launches = ctx->prof_n[k];
      if (total_ms) *total_ms = ctx->prof_ms[k];
      return PHX_OK;
    }
  return set_err(PHX_ENOTFOUND, std::string("unknown kernel kind ") + kind);
}

int phx_profile_reset(phx_context ctx) {
  if (!ctx) return set_err(PHX_EINVAL, "ctx is NULL");
  TRY(collect_events(ctx));
  for (int k = 0; k < K_COUNT; ++k) { ctx->prof_ms[k] = 0; ctx->prof_n[k] = 0; }
  if (ctx->d_algo) CU(cudaMemsetAsync(ctx->d_algo, 0, sizeof(double) * K_COUNT, ctx->stream));
  ctx->launches = 0;
  return PHX_OK;
}

int64_t phx_kernel_launches(phx_context ctx) { return ctx ? ctx->launches : -1; }

int phx_timer_mark(phx_context ctx, int32_t slot) {
  if (!ctx || slot < 0 || slot >= 16) return set_err(PHX_EINVAL, "bad timer slot");
  if (!ctx->marks[slot]) CU(cudaEventCreate(&ctx->marks[slot]));
  CU(cudaEventRecord(ctx->marks[slot], ctx->stream));
  return PHX_OK;
}

int phx_timer_elapsed(phx_context ctx, int32_t a, int32_t b, double* ms) {
  if (!ctx || !ms || a < 0 || a >= 16 || b < 0 || b >= 16 || !ctx->marks[a] || !ctx->marks[b])
    return set_err(PHX_EINVAL, "bad timer slots");
  CU(cudaEventSynchronize(ctx->marks[b]));
  float f = 0;
  CU(cudaEventElapsedTime(&f, ctx->marks[a], ctx->marks[b]));
  *ms = f;
  return PHX_OK;
}

}  // extern "C"
