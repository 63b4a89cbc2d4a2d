// Batched form: the MO vgl of many molecules of uneven size in one pass over the GPU.
//
// Each member is an ordinary context (its tables, coefficients, points and result caches);
// the batch adds one launch per stage that covers every member:
//   1. point order      3 kernels over all points (Morton keys, per-molecule scan, scatter)
//   2. fused AO kernel  persistent; warps take (molecule, 32 points, nucleus chunk) tasks from a
//                       global counter, heaviest molecules first, so uneven sizes balance
//   3. MO contraction   persistent; FP64: DMMA CTA tiles of every molecule from a counter,
//                       longest K first; split-BF16: the tcgen05 kernel over a job list
// The stage sequence is captured once into a CUDA graph and replayed while the members' shapes
// and buffers stay the same. Launch parameters (task granularity of stage 2, CTA tile of the
// FP64 contraction, column tile of the split one) come from an autotuner that times the
// candidates on the batch itself. The reference evaluates one context per call
// (src/qmckl_mo.cpp:114-181 of qmckl_sycl); every per-molecule result here is the one the
// single-context path computes, bit for bit, whatever the tuning.
#include <algorithm>
#include <array>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <fstream>
#include <map>
#include <sstream>

#include "internal.hpp"

namespace qg {
namespace {

constexpr uint64_t kBatchTag = 0xBA7C4EDull;

struct TuneParams {
  int32_t v[3] = {-1, -1, -1};
};

}  // namespace
}  // namespace qg

struct qmckl_batch_struct_device {
  uint64_t tag = qg::kBatchTag;
  std::vector<qmckl_context_device> handles;
  std::vector<qg::Ctx*> members;
  int32_t precision = QMCKL_PRECISION_FP64_DEVICE;
  bool use_graph = true;
  bool async = false;
  bool pinned = false;  // tuning set by the caller
  qg::TuneParams tune;

  // device descriptors, counters and scratch (owned by the batch)
  void* dmem = nullptr;
  size_t dcap = 0;
  size_t off_ao_args = 0, off_ao_begin = 0, off_order = 0, off_point_begin = 0, off_gemm = 0, off_gemm_begin = 0,
         off_split = 0, off_counts = 0, off_counter64 = 0, off_counter32 = 0, off_err = 0;
  int n_ao = 0, n_order = 0, n_gemm = 0;
  int64_t ao_tasks = 0, total_points = 0;
  int gemm_tiles = 0, ao_grid = 0;
  bool high_l = false;  // some member has shells with l >= 4
  int ent_cap = 0;       // largest shared-exponential buffer of a member (0: none shares)
  std::vector<uintptr_t> sig;
  cudaGraph_t graph = nullptr;
  cudaGraphExec_t exec = nullptr;
  cudaEvent_t join = nullptr;
  int64_t launches_per_run = 0;
};

namespace qg {
namespace {

using Batch = qmckl_batch_struct_device;

Batch* batch_of(qmckl_batch_device b) {
  Batch* p = reinterpret_cast<Batch*>(b);
  if (!p || p->tag != kBatchTag) return nullptr;
  return p;
}

size_t align256(size_t x) { return (x + 255) / 256 * 256; }

void drop_graph(Batch* b) {
  if (b->exec) cudaGraphExecDestroy(b->exec);
  if (b->graph) cudaGraphDestroy(b->graph);
  b->exec = nullptr;
  b->graph = nullptr;
}

// ---------------------------------------------------------------- tuning cache
std::mutex g_tune_mutex;
std::map<std::string, TuneParams> g_tune_cache;
bool g_tune_loaded = false;

const char* tune_file() {
  const char* f = std::getenv("QMCKL_GB300_TUNE_CACHE");
  return (f && *f) ? f : nullptr;
}

void load_tune_file() {
  if (g_tune_loaded) return;
  g_tune_loaded = true;
  const char* f = tune_file();
  if (!f) return;
  std::ifstream in(f);
  std::string key;
  TuneParams t;
  while (in >> key >> t.v[0] >> t.v[1] >> t.v[2]) g_tune_cache[key] = t;
}

void store_tune(const std::string& key, const TuneParams& t) {
  g_tune_cache[key] = t;
  const char* f = tune_file();
  if (!f) return;
  std::ofstream out(f, std::ios::app);
  out << key << ' ' << t.v[0] << ' ' << t.v[1] << ' ' << t.v[2] << '\n';
}

// Shape key of a batch: precision, SM count and every member's (points, AOs, MOs, primitives),
// hashed (FNV-1a) to 16 hex digits.
std::string shape_key(const Batch* b) {
  uint64_t h = 1469598103934665603ull;
  auto mix = [&](int64_t v) {
    for (int i = 0; i < 8; ++i) {
      h ^= (uint64_t)((v >> (8 * i)) & 0xff);
      h *= 1099511628211ull;
    }
  };
  int dev = 0, sms = 0;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  cudaGetLastError();
  mix(b->precision);
  mix(sms);
  mix((int64_t)b->members.size());
  for (const Ctx* m : b->members) {
    mix(m->point.num);
    mix(m->ao_basis.ao_num);
    mix(m->mo_basis.mo_num);
    mix(m->ao_basis.prim_num);
  }
  char buf[40];
  snprintf(buf, sizeof buf, "v1-%016llx", (unsigned long long)h);
  return buf;
}

// ---------------------------------------------------------------- plan
struct Member {
  Ctx* ctx;
  int64_t P, A, M, kp;
  double* ao_vgl;
  void* planes;
  double* mo_vgl;
};

// Prepares every member (tables, buffers, coefficient planes) and returns them; members with
// no points or no MOs are left out of the launches.
qmckl_exit_code_device prepare_members(Batch* b, std::vector<Member>& out) {
  const char* fn = "qmckl_batch_provide_mo_vgl_device";
  const qmckl_context_device lead = b->handles[0];
  const bool split = b->precision == QMCKL_PRECISION_SPLIT_BF16_DEVICE;
  out.clear();
  for (size_t i = 0; i < b->members.size(); ++i) {
    Ctx* m = b->members[i];
    const qmckl_context_device h = b->handles[i];
    if (!m->ao_basis.provided || !m->mo_basis.provided)
      return fail(lead, QMCKL_NOT_PROVIDED_DEVICE, fn, "a member has no AO or MO basis");
    qmckl_exit_code_device rc = ensure_tables(m, h);
    if (rc != QMCKL_SUCCESS_DEVICE) return fail(lead, rc, fn, "a member's AO tables could not be built");
    Member e{};
    e.ctx = m;
    e.P = m->point.num;
    e.A = m->ao_basis.ao_num;
    e.M = m->mo_basis.mo_num;
    if (e.P <= 0 || e.M <= 0 || e.A <= 0) continue;
    if (5 * e.P > (int64_t)INT32_MAX - 256) return fail(lead, QMCKL_FAILURE_DEVICE, fn, "a member has too many points");
    AoBasisData& ao = m->ao_basis;
    void* perm = ao.point_perm;
    void* keys = ao.point_keys;
    if (!ensure_raw(m, &perm, &ao.perm_cap, sizeof(int32_t) * e.P) ||
        !ensure_raw(m, &keys, &ao.keys_cap, sizeof(int32_t) * e.P)) {
      ao.point_perm = static_cast<int32_t*>(perm);
      ao.point_keys = static_cast<int32_t*>(keys);
      return fail(lead, QMCKL_ALLOCATION_FAILED_DEVICE, fn, "point order buffers");
    }
    ao.point_perm = static_cast<int32_t*>(perm);
    ao.point_keys = static_cast<int32_t*>(keys);
    MoBasisData& mo = m->mo_basis;
    if (!ensure(m, &mo.mo_vgl, &mo.mo_vgl_cap, sizeof(double) * 5 * e.M * e.P))
      return fail(lead, QMCKL_ALLOCATION_FAILED_DEVICE, fn, "mo_vgl");
    e.mo_vgl = mo.mo_vgl;
    if (split) {
      e.kp = split_k_pad(e.A);
      rc = split_prepare_coef(m, h, e.kp);
      if (rc != QMCKL_SUCCESS_DEVICE) return fail(lead, rc, fn, "coefficient planes");
      e.planes = split_a_planes(m, 5 * ((e.P + 63) / 64 * 64), e.kp);
      if (!e.planes) return fail(lead, QMCKL_ALLOCATION_FAILED_DEVICE, fn, "AO planes");
    } else {
      if (!ensure(m, &ao.ao_vgl, &ao.ao_vgl_cap, sizeof(double) * 5 * e.A * e.P))
        return fail(lead, QMCKL_ALLOCATION_FAILED_DEVICE, fn, "ao_vgl");
      e.ao_vgl = ao.ao_vgl;
    }
    out.push_back(e);
  }
  return QMCKL_SUCCESS_DEVICE;
}

std::vector<uintptr_t> signature_of(const Batch* b, const std::vector<Member>& ms) {
  std::vector<uintptr_t> s;
  s.push_back((uintptr_t)b->precision);
  for (int i = 0; i < 3; ++i) s.push_back((uintptr_t)(intptr_t)b->tune.v[i]);
  for (const Member& e : ms) {
    const Ctx* m = e.ctx;
    s.push_back((uintptr_t)m);
    s.push_back((uintptr_t)m->point.coord);
    s.push_back((uintptr_t)e.P);
    s.push_back((uintptr_t)e.A);
    s.push_back((uintptr_t)e.M);
    s.push_back((uintptr_t)e.ao_vgl);
    s.push_back((uintptr_t)e.planes);
    s.push_back((uintptr_t)e.mo_vgl);
    s.push_back((uintptr_t)m->mo_basis.coefficient_t);
    s.push_back((uintptr_t)m->mo_basis.coef_split);
    s.push_back((uintptr_t)m->ao_basis.tables.nuclei);
    s.push_back((uintptr_t)m->ao_basis.point_perm);
    s.push_back((uintptr_t)m->ao_basis.point_keys);
  }
  return s;
}

// Builds the descriptor arrays for the current tuning and uploads them (synchronously).
qmckl_exit_code_device build_descriptors(Batch* b, const std::vector<Member>& ms) {
  const char* fn = "qmckl_batch_provide_mo_vgl_device";
  const qmckl_context_device lead = b->handles[0];
  const bool split = b->precision == QMCKL_PRECISION_SPLIT_BF16_DEVICE;
  const int n = (int)ms.size();

  // stage 1: point order (members in their own order)
  std::vector<OrderDesc> order(n);
  std::vector<int64_t> point_begin(n + 1, 0);
  for (int i = 0; i < n; ++i) {
    const Member& e = ms[i];
    const AoTables& t = e.ctx->ao_basis.tables;
    OrderDesc& d = order[i];
    d.coord = e.ctx->point.coord;
    d.point_num = e.P;
    d.point_begin = point_begin[i];
    for (int k = 0; k < 3; ++k) d.origin[k] = t.grid_origin[k];
    d.inv_cell = t.grid_inv_cell;
    d.keys = e.ctx->ao_basis.point_keys;
    d.perm = e.ctx->ao_basis.point_perm;
    point_begin[i + 1] = point_begin[i] + e.P;
  }

  // stage 2: AO tasks, molecules with the costliest tasks first
  std::vector<FusedArgs> args(n);
  std::vector<double> task_cost(n);
  b->high_l = false;
  b->ent_cap = 0;
  for (int i = 0; i < n; ++i) {
    const Member& e = ms[i];
    const AoTables& t = e.ctx->ao_basis.tables;
    if (t.lmax > 3) b->high_l = true;

    const int level = b->tune.v[0] < 0 ? 0 : std::min(b->tune.v[0], ao_level_count(t) - 1);
    args[i] = make_fused_args(t, level, e.ctx->point.coord, e.ctx->ao_basis.point_perm, e.P, e.ao_vgl, e.planes,
                              split ? e.kp : e.A);
    if (args[i].ent) b->ent_cap = std::max(b->ent_cap, args[i].ent_cap);
    task_cost[i] = ((double)t.prim_num + 0.5 * (double)t.ao_num) / (double)args[i].chunk_num;
  }
  std::vector<int> ao_order(n);
  for (int i = 0; i < n; ++i) ao_order[i] = i;
  std::stable_sort(ao_order.begin(), ao_order.end(), [&](int x, int y) { return task_cost[x] > task_cost[y]; });
  std::vector<FusedArgs> ao_args(n);
  std::vector<int64_t> ao_begin(n + 1, 0);
  for (int i = 0; i < n; ++i) {
    ao_args[i] = args[ao_order[i]];
    ao_begin[i + 1] = ao_begin[i] + ao_args[i].task_num;
  }

  // stage 3: contraction jobs, longest K first
  std::vector<int> g_order(n);
  for (int i = 0; i < n; ++i) g_order[i] = i;
  std::stable_sort(g_order.begin(), g_order.end(), [&](int x, int y) { return ms[x].A > ms[y].A; });
  std::vector<GemmJob> gemm;
  std::vector<int32_t> gemm_begin(1, 0);
  std::vector<unsigned char> split_jobs;
  const size_t jb = split_job_bytes();
  int64_t tiles = 0;
  if (split) {
    split_jobs.assign(jb * (size_t)n, 0);
    const int n_cap = b->tune.v[2] < 0 ? 160 : b->tune.v[2];
    for (int i = 0; i < n; ++i) {
      const Member& e = ms[g_order[i]];
      const int t = split_make_job_mn(split_jobs.data() + jb * i, e.planes, (e.P + 63) / 64 * 64, e.P,
                                      e.ctx->ao_basis.point_perm, e.ctx->mo_basis.coef_split, e.M, e.kp, e.mo_vgl,
                                      (int)tiles, n_cap);
      if (t < 0) return fail(lead, QMCKL_FAILURE_DEVICE, fn, "cuTensorMapEncodeTiled failed");
      tiles += t;
    }
  } else {
    int tr = 64, tc = 64;
    gemm_shape_tile(b->tune.v[1] < 0 ? 0 : b->tune.v[1], &tr, &tc);
    for (int i = 0; i < n; ++i) {
      const Member& e = ms[g_order[i]];
      GemmJob j{};
      j.a = e.ao_vgl;
      j.b = e.ctx->mo_basis.coefficient_t;
      j.c = e.mo_vgl;
      j.rows = 5 * e.P;
      j.k = e.A;
      j.cols = e.M;
      j.col_tiles = (int32_t)((e.M + tc - 1) / tc);
      j.tile_begin = (int32_t)tiles;
      tiles += ((j.rows + tr - 1) / tr) * j.col_tiles;
      gemm.push_back(j);
      gemm_begin.push_back((int32_t)tiles);
    }
  }
  if (tiles > (int64_t)INT32_MAX / 2) return fail(lead, QMCKL_FAILURE_DEVICE, fn, "batch too large");

  // one device block: descriptors, counters, per-molecule cell counters
  size_t off = 0;
  auto take = [&](size_t bytes) {
    const size_t o = off;
    off = align256(off + std::max<size_t>(bytes, 1));
    return o;
  };
  b->off_order = take(sizeof(OrderDesc) * n);
  b->off_point_begin = take(sizeof(int64_t) * (n + 1));
  b->off_ao_args = take(sizeof(FusedArgs) * n);
  b->off_ao_begin = take(sizeof(int64_t) * (n + 1));
  b->off_gemm = take(split ? jb * n : sizeof(GemmJob) * n);
  b->off_gemm_begin = take(sizeof(int32_t) * (n + 1));
  b->off_counter64 = take(sizeof(unsigned long long));
  b->off_counter32 = take(sizeof(unsigned int));
  b->off_err = take(sizeof(int));
  b->off_counts = take(sizeof(int32_t) * (size_t)kOrderCells * (size_t)std::max(n, 1));
  const size_t total = off;
  if (total > b->dcap) {
    drop_graph(b);
    if (b->dmem) cudaFree(b->dmem);
    b->dmem = nullptr;
    b->dcap = 0;
    if (cudaMalloc(&b->dmem, total) != cudaSuccess) {
      cudaGetLastError();
      return fail(lead, QMCKL_ALLOCATION_FAILED_DEVICE, fn, "batch descriptors");
    }
    b->dcap = total;
  }
  std::vector<unsigned char> host(b->off_counts, 0);  // descriptors, zeroed counters and error word
  auto put = [&](size_t o, const void* src, size_t bytes) {
    if (bytes) memcpy(host.data() + o, src, bytes);
  };
  put(b->off_order, order.data(), sizeof(OrderDesc) * n);
  put(b->off_point_begin, point_begin.data(), sizeof(int64_t) * (n + 1));
  put(b->off_ao_args, ao_args.data(), sizeof(FusedArgs) * n);
  put(b->off_ao_begin, ao_begin.data(), sizeof(int64_t) * (n + 1));
  if (split) {
    put(b->off_gemm, split_jobs.data(), jb * n);
    std::vector<int32_t> sb(n + 1, 0);  // unused by the split kernel (its jobs hold their first tile)
    put(b->off_gemm_begin, sb.data(), sizeof(int32_t) * (n + 1));
  } else {
    put(b->off_gemm, gemm.data(), sizeof(GemmJob) * n);
    put(b->off_gemm_begin, gemm_begin.data(), sizeof(int32_t) * (n + 1));
  }
  if (cudaMemcpy(b->dmem, host.data(), host.size(), cudaMemcpyHostToDevice) != cudaSuccess) {
    cudaGetLastError();
    return fail(lead, QMCKL_FAILURE_DEVICE, fn, "descriptor upload failed");
  }
  b->n_order = b->n_ao = b->n_gemm = n;
  b->total_points = point_begin[n];
  b->ao_tasks = ao_begin[n];
  b->gemm_tiles = (int)tiles;
  b->ao_grid = ao_batch_resident_ctas(split, b->high_l, b->ent_cap);
  return QMCKL_SUCCESS_DEVICE;
}

template <class T>
T* at(const Batch* b, size_t off) {
  return reinterpret_cast<T*>(static_cast<unsigned char*>(b->dmem) + off);
}

cudaError_t stage_order(Batch* b, cudaStream_t s) {
  return launch_order_batch(s, at<OrderDesc>(b, b->off_order), at<int64_t>(b, b->off_point_begin), b->n_order,
                            b->total_points, at<int32_t>(b, b->off_counts));
}

cudaError_t stage_ao(Batch* b, cudaStream_t s) {
  return launch_ao_batch(s, b->precision == QMCKL_PRECISION_SPLIT_BF16_DEVICE, b->high_l, b->ent_cap,
                         at<FusedArgs>(b, b->off_ao_args),
                         at<int64_t>(b, b->off_ao_begin), b->n_ao, b->ao_tasks,
                         at<unsigned long long>(b, b->off_counter64), b->ao_grid);
}

cudaError_t stage_mo(Batch* b, cudaStream_t s) {
  if (b->n_gemm == 0 || b->gemm_tiles == 0) return cudaSuccess;
  if (b->precision == QMCKL_PRECISION_SPLIT_BF16_DEVICE) {
    cudaError_t e = cudaMemsetAsync(at<int>(b, b->off_err), 0, sizeof(int), s);
    if (e != cudaSuccess) return e;
    return split_launch_jobs(s, at<unsigned char>(b, b->off_gemm), b->n_gemm, b->gemm_tiles, at<int>(b, b->off_err));
  }
  return launch_dgemm_batch(s, b->tune.v[1] < 0 ? 0 : b->tune.v[1], true, at<GemmJob>(b, b->off_gemm),
                            at<int32_t>(b, b->off_gemm_begin), b->n_gemm, b->gemm_tiles,
                            at<unsigned int>(b, b->off_counter32));
}

int64_t kernels_per_run(const Batch* b) {
  int64_t k = 0;
  if (b->total_points > 0) k += 3;
  if (b->ao_tasks > 0) k += 1;
  if (b->gemm_tiles > 0) k += 1;
  return k;
}

cudaError_t run_stages(Batch* b, cudaStream_t s, bool profile) {
  Ctx* lead = b->members[0];
  cudaError_t e;
  const bool split = b->precision == QMCKL_PRECISION_SPLIT_BF16_DEVICE;
  if (profile) {
    {
      LaunchScope scope(lead, "batch_point_order");
      lead->launch_count += 2;  // three kernels
      e = stage_order(b, s);
    }
    if (e != cudaSuccess) return e;
    {
      LaunchScope scope(lead, split ? "batch_ao_vgl_bf16_planes" : "batch_ao_vgl");
      e = stage_ao(b, s);
    }
    if (e != cudaSuccess) return e;
    LaunchScope scope(lead, split ? "batch_mo_vgl_split_bf16" : "batch_mo_vgl_dgemm");
    return stage_mo(b, s);
  }
  e = stage_order(b, s);
  if (e == cudaSuccess) e = stage_ao(b, s);
  if (e == cudaSuccess) e = stage_mo(b, s);
  return e;
}

// Times one stage (ms, best of reps after one warm-up) on the lead stream.
double time_stage(Batch* b, cudaError_t (*stage)(Batch*, cudaStream_t), int reps) {
  cudaStream_t s = b->members[0]->stream;
  cudaEvent_t e0, e1;
  cudaEventCreate(&e0);
  cudaEventCreate(&e1);
  double best = 1e300;
  stage(b, s);
  for (int r = 0; r < reps; ++r) {
    cudaEventRecord(e0, s);
    stage(b, s);
    cudaEventRecord(e1, s);
    cudaEventSynchronize(e1);
    float ms = 0.f;
    cudaEventElapsedTime(&ms, e0, e1);
    best = std::min(best, (double)ms);
  }
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  if (cudaGetLastError() != cudaSuccess) return 1e300;
  return best;
}

// Chooses the tuning of each stage by timing its candidates on this batch (stages are
// independent: the AO task granularity does not change the contraction's inputs' layout).
qmckl_exit_code_device autotune(Batch* b, const std::vector<Member>& ms) {
  const bool split = b->precision == QMCKL_PRECISION_SPLIT_BF16_DEVICE;
  int max_level = 0;
  for (const Member& e : ms) max_level = std::max(max_level, ao_level_count(e.ctx->ao_basis.tables) - 1);
  b->tune.v[0] = 0;
  b->tune.v[1] = 0;
  b->tune.v[2] = 160;
  qmckl_exit_code_device rc = build_descriptors(b, ms);
  if (rc != QMCKL_SUCCESS_DEVICE) return rc;
  stage_order(b, b->members[0]->stream);
  // AO task granularity
  int best_level = 0;
  double best = 1e300;
  for (int lv = 0; lv <= std::min(max_level, 4); ++lv) {
    b->tune.v[0] = lv;
    rc = build_descriptors(b, ms);
    if (rc != QMCKL_SUCCESS_DEVICE) return rc;
    const double t = time_stage(b, stage_ao, 3);
    if (t < best * 0.98) {
      best = t;
      best_level = lv;
    }
  }
  b->tune.v[0] = best_level;
  // contraction tile
  best = 1e300;
  if (split) {
    int best_cap = 160;
    const int caps[] = {160, 128, 96, 64};
    for (int cap : caps) {
      b->tune.v[2] = cap;
      rc = build_descriptors(b, ms);
      if (rc != QMCKL_SUCCESS_DEVICE) return rc;
      const double t = time_stage(b, stage_mo, 3);
      if (t < best * 0.98) {
        best = t;
        best_cap = cap;
      }
    }
    b->tune.v[2] = best_cap;
  } else {
    int best_shape = 0;
    for (int shape = 0; shape < kGemmShapes; ++shape) {
      b->tune.v[1] = shape;
      rc = build_descriptors(b, ms);
      if (rc != QMCKL_SUCCESS_DEVICE) return rc;
      const double t = time_stage(b, stage_mo, 2);
      if (t < best * 0.98) {
        best = t;
        best_shape = shape;
      }
    }
    b->tune.v[1] = best_shape;
  }
  if (split && b->tune.v[1] < 0) b->tune.v[1] = 0;
  if (!split) b->tune.v[2] = 160;
  drop_graph(b);
  b->sig.clear();
  return QMCKL_SUCCESS_DEVICE;
}

}  // namespace
}  // namespace qg

using namespace qg;

extern "C" {

qmckl_batch_device qmckl_batch_create_device(const qmckl_context_device* members, int64_t member_num) {
  if (!members || member_num < 1 || member_num > (1 << 20)) return QMCKL_NULL_BATCH_DEVICE;
  std::vector<Ctx*> ms;
  for (int64_t i = 0; i < member_num; ++i) {
    if (qmckl_context_check_device(members[i]) == QMCKL_NULL_CONTEXT_DEVICE) return QMCKL_NULL_BATCH_DEVICE;
    Ctx* c = ctx_of(members[i]);
    if (std::find(ms.begin(), ms.end(), c) != ms.end()) return QMCKL_NULL_BATCH_DEVICE;
    if (c->device_id != ctx_of(members[0])->device_id) return QMCKL_NULL_BATCH_DEVICE;
    ms.push_back(c);
  }
  if (!ensure_device(ms[0])) return QMCKL_NULL_BATCH_DEVICE;
  Batch* b = new Batch;
  b->handles.assign(members, members + member_num);
  b->members = ms;
  return reinterpret_cast<qmckl_batch_device>(b);
}

qmckl_exit_code_device qmckl_batch_destroy_device(qmckl_batch_device batch) {
  Batch* b = batch_of(batch);
  if (!b) return QMCKL_INVALID_CONTEXT_DEVICE;
  cudaSetDevice(b->members[0]->device_id);
  if (b->members[0]->stream) cudaStreamSynchronize(b->members[0]->stream);
  drop_graph(b);
  if (b->join) cudaEventDestroy(b->join);
  if (b->dmem) cudaFree(b->dmem);
  cudaGetLastError();
  b->tag = 0;
  delete b;
  return QMCKL_SUCCESS_DEVICE;
}

qmckl_exit_code_device qmckl_batch_set_precision_mode_device(qmckl_batch_device batch, int32_t mode) {
  Batch* b = batch_of(batch);
  if (!b) return QMCKL_INVALID_CONTEXT_DEVICE;
  if (mode != QMCKL_PRECISION_FP64_DEVICE && mode != QMCKL_PRECISION_SPLIT_BF16_DEVICE)
    return fail(b->handles[0], QMCKL_INVALID_ARG_2_DEVICE, "qmckl_batch_set_precision_mode_device",
                "mode must be QMCKL_PRECISION_FP64_DEVICE or QMCKL_PRECISION_SPLIT_BF16_DEVICE");
  if (b->precision != mode) {
    b->precision = mode;
    if (!b->pinned) b->tune = TuneParams{};
    drop_graph(b);
    b->sig.clear();
    qmckl_batch_touch_device(batch);
  }
  return QMCKL_SUCCESS_DEVICE;
}

qmckl_exit_code_device qmckl_batch_set_graph_device(qmckl_batch_device batch, int32_t enable) {
  Batch* b = batch_of(batch);
  if (!b) return QMCKL_INVALID_CONTEXT_DEVICE;
  b->use_graph = enable != 0;
  return QMCKL_SUCCESS_DEVICE;
}

qmckl_exit_code_device qmckl_batch_set_async_device(qmckl_batch_device batch, int32_t async) {
  Batch* b = batch_of(batch);
  if (!b) return QMCKL_INVALID_CONTEXT_DEVICE;
  b->async = async != 0;
  return QMCKL_SUCCESS_DEVICE;
}

qmckl_exit_code_device qmckl_batch_synchronize_device(qmckl_batch_device batch) {
  Batch* b = batch_of(batch);
  if (!b) return QMCKL_INVALID_CONTEXT_DEVICE;
  Ctx* lead = b->members[0];
  if (cudaStreamSynchronize(lead->stream) != cudaSuccess)
    return fail(b->handles[0], QMCKL_FAILURE_DEVICE, "qmckl_batch_synchronize_device",
                cudaGetErrorString(cudaGetLastError()));
  if (b->precision == QMCKL_PRECISION_SPLIT_BF16_DEVICE && b->dmem) {
    int h = 0;
    cudaMemcpy(&h, at<int>(b, b->off_err), sizeof(int), cudaMemcpyDeviceToHost);
    if (h)
      return fail(b->handles[0], QMCKL_FAILURE_DEVICE, "qmckl_batch_synchronize_device",
                  "split-BF16 GEMM: a pipeline wait timed out");
  }
  return QMCKL_SUCCESS_DEVICE;
}

qmckl_exit_code_device qmckl_batch_touch_device(qmckl_batch_device batch) {
  Batch* b = batch_of(batch);
  if (!b) return QMCKL_INVALID_CONTEXT_DEVICE;
  for (qmckl_context_device h : b->handles) {
    qmckl_exit_code_device rc = qmckl_context_touch_device(h);
    if (rc != QMCKL_SUCCESS_DEVICE) return rc;
  }
  return QMCKL_SUCCESS_DEVICE;
}

qmckl_exit_code_device qmckl_batch_set_tuning_device(qmckl_batch_device batch, const int32_t* params, int64_t n) {
  Batch* b = batch_of(batch);
  if (!b) return QMCKL_INVALID_CONTEXT_DEVICE;
  const char* fn = "qmckl_batch_set_tuning_device";
  if (!params) return fail(b->handles[0], QMCKL_INVALID_ARG_2_DEVICE, fn, "NULL pointer");
  if (n != 3) return fail(b->handles[0], QMCKL_INVALID_ARG_3_DEVICE, fn, "expected 3 parameters");
  if (params[0] < 0 || params[0] > 30 || params[1] < 0 || params[1] >= kGemmShapes || params[2] < 16 ||
      params[2] > 160 || params[2] % 16 != 0)
    return fail(b->handles[0], QMCKL_INVALID_ARG_2_DEVICE, fn, "parameter out of range");
  for (int i = 0; i < 3; ++i) b->tune.v[i] = params[i];
  b->pinned = true;
  drop_graph(b);
  b->sig.clear();
  return QMCKL_SUCCESS_DEVICE;
}

qmckl_exit_code_device qmckl_batch_get_tuning_device(qmckl_batch_device batch, int32_t* params, int64_t n) {
  Batch* b = batch_of(batch);
  if (!b) return QMCKL_INVALID_CONTEXT_DEVICE;
  if (!params) return fail(b->handles[0], QMCKL_INVALID_ARG_2_DEVICE, "qmckl_batch_get_tuning_device", "NULL pointer");
  if (n < 3) return fail(b->handles[0], QMCKL_INVALID_ARG_3_DEVICE, "qmckl_batch_get_tuning_device", "expected 3");
  for (int i = 0; i < 3; ++i) params[i] = b->tune.v[i];
  return QMCKL_SUCCESS_DEVICE;
}

int64_t qmckl_batch_get_launch_count_device(qmckl_batch_device batch) {
  Batch* b = batch_of(batch);
  if (!b) return 0;
  return b->launches_per_run;
}

static qmckl_exit_code_device batch_provide(Batch* b, bool force_tune) {
  const char* fn = "qmckl_batch_provide_mo_vgl_device";
  const qmckl_context_device lead_h = b->handles[0];
  Ctx* lead = b->members[0];
  if (!ensure_device(lead)) return fail(lead_h, QMCKL_FAILURE_DEVICE, fn, "no usable CUDA device");
  bool stale = force_tune;
  for (Ctx* m : b->members) stale = stale || m->point.date > m->mo_basis.mo_vgl_date;
  if (!stale) return QMCKL_SUCCESS_DEVICE;

  std::vector<Member> ms;
  qmckl_exit_code_device rc = prepare_members(b, ms);
  if (rc != QMCKL_SUCCESS_DEVICE) return rc;

  // work queued by members on their own streams (their points) comes first
  if (!b->join) cudaEventCreateWithFlags(&b->join, cudaEventDisableTiming);
  for (Ctx* m : b->members)
    if (m->stream && m->stream != lead->stream) {
      cudaEventRecord(b->join, m->stream);
      cudaStreamWaitEvent(lead->stream, b->join, 0);
    }

  if (!ms.empty()) {
    if (force_tune || (!b->pinned && b->tune.v[0] < 0)) {
      const std::string key = shape_key(b);
      bool found = false;
      if (!force_tune) {
        std::lock_guard<std::mutex> lock(g_tune_mutex);
        load_tune_file();
        auto it = g_tune_cache.find(key);
        if (it != g_tune_cache.end()) {
          b->tune = it->second;
          found = true;
        }
      }
      if (!found) {
        rc = autotune(b, ms);
        if (rc != QMCKL_SUCCESS_DEVICE) return rc;
        std::lock_guard<std::mutex> lock(g_tune_mutex);
        store_tune(key, b->tune);
      }
    }
    std::vector<uintptr_t> sig = signature_of(b, ms);
    if (sig != b->sig) {
      drop_graph(b);
      rc = build_descriptors(b, ms);
      if (rc != QMCKL_SUCCESS_DEVICE) return rc;
      b->sig = sig;
    }
    b->launches_per_run = kernels_per_run(b);
    cudaError_t e = cudaSuccess;
    bool ran = false;
    if (b->use_graph && !lead->profiling) {
      if (!b->exec) {
        // capture once; a stream that cannot be captured (e.g. the legacy default stream)
        // falls back to ordinary launches
        if (cudaStreamBeginCapture(lead->stream, cudaStreamCaptureModeRelaxed) == cudaSuccess) {
          const cudaError_t e2 = run_stages(b, lead->stream, false);
          cudaGraph_t g = nullptr;
          const cudaError_t e3 = cudaStreamEndCapture(lead->stream, &g);
          if (e2 == cudaSuccess && e3 == cudaSuccess && g) {
            b->graph = g;
            if (cudaGraphInstantiate(&b->exec, g, 0) != cudaSuccess) drop_graph(b);
          } else if (g) {
            cudaGraphDestroy(g);
          }
        }
        cudaGetLastError();
      }
      if (b->exec) {
        e = cudaGraphLaunch(b->exec, lead->stream);
        lead->launch_count += b->launches_per_run;
        ran = true;
      }
    }
    if (!ran) e = run_stages(b, lead->stream, true);
    if (e != cudaSuccess) {
      cudaGetLastError();
      drop_graph(b);
      return fail(lead_h, QMCKL_FAILURE_DEVICE, fn, cudaGetErrorString(e));
    }
  }
  if (!b->async) {
    rc = qmckl_batch_synchronize_device(reinterpret_cast<qmckl_batch_device>(b));
    if (rc != QMCKL_SUCCESS_DEVICE) return rc;
  }
  const bool split = b->precision == QMCKL_PRECISION_SPLIT_BF16_DEVICE;
  for (const Member& e : ms) {
    Ctx* m = e.ctx;
    m->mo_basis.mo_vgl_date = m->date;
    m->ao_basis.perm_date = m->point.date;
    if (!split) m->ao_basis.ao_vgl_date = m->date;
  }
  for (Ctx* m : b->members)  // members without points or MOs have nothing to compute
    if (m->point.num <= 0 || m->mo_basis.mo_num <= 0) m->mo_basis.mo_vgl_date = m->date;
  return QMCKL_SUCCESS_DEVICE;
}

qmckl_exit_code_device qmckl_batch_provide_mo_vgl_device(qmckl_batch_device batch) {
  QG_NVTX_RANGE("qmckl_batch_provide_mo_vgl_device");
  Batch* b = batch_of(batch);
  if (!b) return QMCKL_INVALID_CONTEXT_DEVICE;
  for (qmckl_context_device h : b->handles)
    if (qmckl_context_check_device(h) == QMCKL_NULL_CONTEXT_DEVICE) return QMCKL_INVALID_CONTEXT_DEVICE;
  cudaSetDevice(b->members[0]->device_id);
  return batch_provide(b, false);
}

qmckl_exit_code_device qmckl_batch_autotune_device(qmckl_batch_device batch) {
  Batch* b = batch_of(batch);
  if (!b) return QMCKL_INVALID_CONTEXT_DEVICE;
  cudaSetDevice(b->members[0]->device_id);
  b->pinned = false;
  return batch_provide(b, true);
}

}  // extern "C"
