// Internal definitions of the GB300 QMCkl basis-evaluation library: the context
// structure, the packed device tables the fused kernels read, and the launch
// interfaces of the CUDA kernels. Not part of the public ABI (include/qmckl_gpu.h).
#pragma once

#include <cuda_runtime.h>
#include <nvtx3/nvToolsExt.h>

#include <cstdint>
#include <mutex>
#include <string>
#include <unordered_map>
#include <vector>

#include "../../include/qmckl_gpu.h"
#include "bounds.cuh"

namespace qg {

// NVTX range around a C-ABI entry point (header-only NVTX 3: a no-op unless a profiler such as
// ncu or Nsight Systems is attached), so that a timeline shows each call with its kernels.
struct NvtxRange {
  explicit NvtxRange(const char* name) { nvtxRangePushA(name); }
  ~NvtxRange() { nvtxRangePop(); }
  NvtxRange(const NvtxRange&) = delete;
  NvtxRange& operator=(const NvtxRange&) = delete;
};
#define QG_NVTX_RANGE(name) ::qg::NvtxRange qg_nvtx_range_(name)

constexpr uint64_t kValidTag = 0xBEEFFACEull;    // include/qmckl_types.hpp:12 of the reference
constexpr uint64_t kInvalidTag = 0xDEADBEEFull;  // include/qmckl_types.hpp:13
// -ln(1e-12): screening cutoff hard-coded by the reference (src/qmckl_ao_sycl.cpp:22,117,449).
constexpr double kCutoff = 27.631021115928547;
// Largest angular momentum handled; the reference's lstart table has 21 entries
// (src/qmckl_ao_sycl.cpp:161), i.e. l + 1 <= 20.
constexpr int kMaxL = 19;

// ---- Packed tables read by the fused AO kernels (built on the host at finalize) ----
// Nuclei are visited in index order and, within a nucleus, its shells in index order;
// this is the order in which the reference numbers AOs (src/qmckl_ao_sycl.cpp:166-188).
struct NucleusEntry {      // 64 bytes
  double x, y, z;          // nucleus coordinates
  uint64_t screen_bits;    // bit pattern of fl(cutoff * nucleus_range): a point is screened for
                           // this nucleus iff bits(r2) > screen_bits (non-negative doubles order
                           // like their bit patterns), the reference's test at ao_sycl.cpp:53
  int32_t shell_begin, shell_end;  // range in the packed shell list
  int32_t ao_begin, ao_end;        // AO columns of this nucleus
  int32_t lmax;
  int32_t ent_begin, ent_num;      // distinct exponents of the nucleus in AoTables::ent
  int32_t pad;
};
struct ShellEntry {        // 16 bytes
  int32_t prim_begin, prim_end;  // range in the packed primitive list
  int32_t ao_begin;
  int16_t l;
  int16_t unit_aof;        // 1: every AO factor of the shell is exactly 1 (the kernels load none)
};
struct PrimEntry {         // 48 bytes
  double expo;
  double coef;             // coefficient_normalized = coefficient * prim_factor * shell_factor
  double m2a;              // -2 * expo (exact)
  double m2a2;             // -2 * expo^2
  uint64_t thr_bits;       // bits of the smallest r2 with fl(expo * r2) > cutoff: the primitive
                           // is skipped iff bits(r2) >= thr_bits (ao_sycl.cpp:72-75)
  int32_t ent;             // index of its exponent among the nucleus' distinct exponents
  int32_t pad;
};

// A contiguous group of nuclei processed by one warp task.
struct NucleusChunk {
  int32_t nucl_begin, nucl_end;
  int32_t ao_begin, ao_end;
  int32_t shell_lo, shell_hi;  // packed shells evaluated: all of the nuclei's, or part of one nucleus's
};

// 2^(j/32), j = 0..31, as hi + lo doubles (hi = the double nearest to the value): the table of
// the AO kernel's exponential (table-driven method of P. T. P. Tang, ACM TOMS 15(2), 1989).
// fine[j] = 2^(j/kFine) as an FP32 pair (x = the float nearest to the value, y = the float
// nearest to the remainder: 48 significant bits), the table of the split-BF16 form's primitives.
constexpr int kFineBits = 10;
constexpr int kFine = 1 << kFineBits;
struct ExpTable {
  double hi[32];
  double lo[32];
  float2 fine[kFine];
};

// A primitive of the packed list prepared for the split-BF16 form's radials, which evaluate
// v = coef * e^(-expo r2) in FP32 pair arithmetic as sign * 2^k * e^y with
// y = ln(mant) - expo r2, |coef| = mant * 2^k, mant in [1, 2): the coefficient folds into the
// exponential. ln(mant) = jm * L + dh with L = ln 2 / kFine, so that jm joins the table index.
// Also the distinct exponents of a nucleus (shared exponentials, coefficient 1). 32 bytes, so
// that the medium basis's list (2123 primitives, 68 KB) stays in L1 beside the other tables.
struct PrimFold {
  uint64_t thr_bits;       // PrimEntry::thr_bits, or 0 (never active) for a zero coefficient
  float nah, nal;          // -expo as an FP32 pair (nah + nal = -expo to 48 bits)
  float dh;                // ln(mant) - jm L, |dh| <= L / 2
  uint32_t jeb;            // jm (nearest integer to ln(mant) / L, in [0, kFine]) in bits 0..11,
                           // sign * 2^k as float bits (sign, biased exponent) in bits 23..31
  union {
    struct {
      float ch, cl;        // a primitive: coef as an FP32 pair (shared exponentials: v = coef * e)
    } c;
    double na;             // a distinct exponent: -expo (the FP64 outputs' shared exponentials)
  };
};
static_assert(sizeof(PrimFold) == 32, "PrimFold is 32 bytes");
constexpr uint32_t kFoldJmMask = 0xFFFu;


struct AoTables {
  NucleusEntry* nuclei = nullptr;   // [nucl_num]
  ShellEntry* shells = nullptr;     // [shell_num] packed
  PrimEntry* prims = nullptr;       // [prim_num] packed
  double* ao_factor = nullptr;      // [ao_num]
  int32_t* shell_orig = nullptr;    // packed shell -> user shell index
  int32_t* shell_nucl = nullptr;    // packed shell -> nucleus
  int32_t* prim_orig = nullptr;     // packed primitive -> user primitive index
  bool prims_unique = true;         // no user primitive is shared by two shells
  NucleusChunk* chunks = nullptr;   // all chunk levels, concatenated
  // Level v splits the nuclei into level_sizes[v] chunks of balanced cost, stored at
  // chunks + level_offsets[v]; the launch picks the level that fills the GPU.
  std::vector<int32_t> level_offsets, level_sizes;
  // Pieces: every nucleus's shells cut into consecutive ranges of about a quarter of a nucleus's
  // average cost, one chunk each, at chunks + piece_offset (after the levels; the finest tasks of
  // the forward AO kernel's last segment).
  int32_t piece_offset = 0, piece_num = 0;
  ExpTable* exp_table = nullptr;    // device copy of the exponential's table
  // [prim_num] packed, or null when some exponent or coefficient is outside the FP32 folded
  // evaluation's range (then the split-BF16 form evaluates its radials like the FP64 form)
  PrimFold* fold = nullptr;
  // Distinct exponents per nucleus (NucleusEntry::ent_begin/ent_num), as PrimFold entries with
  // coefficient 1, when the basis repeats exponents within nuclei enough for the kernels to
  // evaluate each exponential once per nucleus and share it between shells (null otherwise).
  PrimFold* ent = nullptr;
  int32_t ent_cap = 0;              // largest distinct-exponent count of a nucleus
  bool ent_forced = false;          // sharing requested explicitly (else: FP64 outputs only)
  // grid for grouping points into spatially coherent warps: 32 cells per axis over the
  // nuclei's bounding box plus a margin (points outside are clamped to the border cells)
  double grid_origin[3] = {0, 0, 0};
  double grid_inv_cell = 1.0;
  int32_t nucl_num = 0, shell_num = 0, prim_num = 0, ao_num = 0, lmax = 0;
  int sm_count = 152;
  bool valid = false;
  std::vector<NucleusEntry> h_nuclei;
  std::vector<ShellEntry> h_shells;
  std::vector<PrimEntry> h_prims;
  std::vector<PrimFold> h_fold, h_ent;
  std::vector<NucleusChunk> h_chunks;
  std::vector<int32_t> h_shell_orig, h_shell_nucl, h_prim_orig;
  std::vector<double> h_ao_factor;
};

struct PointData {
  int64_t num = 0;
  uint64_t date = 0;
  double* coord = nullptr;  // [3][num] (the reference's ctx->point.coord, Fortran (num,3))
};

struct WalkerData {
  int64_t num = 0;
  PointData point;
};

struct ElectronData {
  int64_t num = 0, up_num = 0, down_num = 0;
  WalkerData walker, walker_old;
  // cached distances (src/qmckl_electron.cpp:192-296 of the reference)
  double* en_distance = nullptr;
  size_t en_distance_cap = 0;
  uint64_t en_distance_date = 0;
  double* ee_distance = nullptr;
  size_t ee_distance_cap = 0;
  uint64_t ee_distance_date = 0;
  int32_t uninitialized = 0;
  bool provided = false;
};

struct NucleusData {
  int64_t num = 0;
  double* charge = nullptr;  // [num]
  double* coord = nullptr;   // [3][num]
  int32_t uninitialized = 0;
  bool provided = false;
};

struct AoBasisData {
  char type = 0;
  int64_t shell_num = 0, prim_num = 0, ao_num = 0;
  int64_t* nucleus_index = nullptr;
  int64_t* nucleus_shell_num = nullptr;
  int32_t* shell_ang_mom = nullptr;
  int64_t* shell_prim_num = nullptr;
  int64_t* shell_prim_index = nullptr;
  double* shell_factor = nullptr;
  double* exponent = nullptr;
  double* coefficient = nullptr;
  double* prim_factor = nullptr;
  double* ao_factor = nullptr;
  // derived at finalize (src/qmckl_ao_sycl.cpp:1087-1231)
  int64_t* nucleus_prim_index = nullptr;
  double* coefficient_normalized = nullptr;
  int32_t* nucleus_max_ang_mom = nullptr;
  double* nucleus_range = nullptr;
  // per-nucleus sorted, merged exponent tables (src/qmckl_ao_sycl.cpp:855-1065)
  int32_t* prim_num_per_nucleus = nullptr;  // [nucl_num]
  double* expo_per_nucleus = nullptr;       // [nucl_num][hpc_prim_max]
  double* coef_per_nucleus = nullptr;       // [nucl_num][hpc_shell_max][hpc_prim_max]
  int64_t hpc_prim_max = 0, hpc_shell_max = 0;
  AoTables tables;
  // caches
  double* shell_vgl = nullptr;
  size_t shell_vgl_cap = 0;
  uint64_t shell_vgl_date = 0;
  double* ao_vgl = nullptr;
  size_t ao_vgl_cap = 0;
  uint64_t ao_vgl_date = 0;
  double* ao_value = nullptr;
  size_t ao_value_cap = 0;
  uint64_t ao_value_date = 0;
  // processing order of the current points (see launch_point_order), valid for perm_date
  int32_t* point_perm = nullptr;
  int32_t* point_keys = nullptr;
  int32_t* cell_counts = nullptr;
  size_t perm_cap = 0, keys_cap = 0, counts_cap = 0;
  uint64_t perm_date = 0;
  int32_t uninitialized = 0;
  bool provided = false;
};

// The host-buffer path's contraction jobs (one per point range), kept on the device while the
// shape and buffers they were encoded for stay the same.
constexpr int kMaxHostChunks = 64;
struct HostChunkKey {
  int64_t P = 0, M = 0, kp = 0;
  int chunks = 0;
  double ratio = 0.0;
  const void *a_planes = nullptr, *b_planes = nullptr, *out = nullptr, *perm = nullptr;
  bool operator==(const HostChunkKey& o) const {
    return P == o.P && M == o.M && kp == o.kp && chunks == o.chunks && ratio == o.ratio && a_planes == o.a_planes &&
           b_planes == o.b_planes && out == o.out && perm == o.perm;
  }
};
struct HostChunkJobs {
  HostChunkKey key;
  void* jobs = nullptr;  // device copy of the SplitJob list
  size_t jobs_cap = 0;
  int tiles[kMaxHostChunks] = {};
};

struct MoBasisData {
  int64_t mo_num = 0;
  double* coefficient = nullptr;    // [mo_num][ao_num]
  double* coefficient_t = nullptr;  // [ao_num][mo_num]
  double* mo_vgl = nullptr;
  size_t mo_vgl_cap = 0;
  uint64_t mo_vgl_date = 0;
  double* mo_value = nullptr;
  size_t mo_value_cap = 0;
  uint64_t mo_value_date = 0;
  // split-BF16 form: the coefficient split into three BF16 planes (hi, mid, lo), each
  // [mo_pad][ao_pad] K-major, and the AO operand planes for the current points.
  void* coef_split = nullptr;
  int64_t split_mo_pad = 0, split_ao_pad = 0;
  void* ao_split = nullptr;
  size_t ao_split_cap = 0;
  void* split_job = nullptr;  // device copy of the contraction's job descriptor
  size_t split_job_cap = 0;
  HostChunkJobs host_jobs;    // the host-buffer path's job list
  int32_t uninitialized = 0;
  bool provided = false;
};

struct KernelStat {
  std::string name;
  int64_t launches = 0;
  double total_ms = 0.0;
};
struct PendingEvent {
  int slot;
  cudaEvent_t start, stop;
};

}  // namespace qg

struct qmckl_error_struct_device {
  qmckl_exit_code_device exit_code = 0;
  char function[QMCKL_MAX_FUN_LEN_DEVICE] = {0};
  char message[QMCKL_MAX_MSG_LEN_DEVICE] = {0};
};

struct qmckl_context_struct_device {
  uint64_t tag = qg::kValidTag;
  int32_t device_id = 0;
  cudaStream_t stream = nullptr;
  bool own_stream = false;
  cudaStream_t copy_stream = nullptr;  // device-to-host copies overlapped with compute
  cudaEvent_t chunk_done[qg::kMaxHostChunks] = {};  // host-buffer path: range k computed
  bool async = false;
  int32_t precision = QMCKL_PRECISION_FP64_DEVICE;
  int32_t shared_exp = QMCKL_SHARED_EXP_AUTO_DEVICE;  // shared exponentials of the AO kernels

  std::recursive_mutex mutex;
  int lock_count = 0;
  qmckl_error_struct_device error;

  // allocation registries (src/qmckl_memory.cpp:15-220 of the reference)
  std::unordered_map<void*, size_t> device_allocs;
  std::unordered_map<void*, size_t> host_allocs;
  int64_t fail_alloc_countdown = 0;

  uint64_t date = 0;
  qg::PointData point;
  qg::NucleusData nucleus;
  qg::ElectronData electron;
  qg::AoBasisData ao_basis;
  qg::MoBasisData mo_basis;

  // grow-only scratch for layout changes of host inputs (points, nuclei)
  void* staging = nullptr;
  size_t staging_cap = 0;
  // grow-only scratch of the adjoint (vector-Jacobian) calls
  void* vjp_buf = nullptr;
  size_t vjp_cap = 0;
  // task counter of the persistent AO kernels (zeroed before each launch)
  unsigned long long* task_counter = nullptr;
  // failure-handling test hook of the split-BF16 contraction (qmckl_set_split_wait_test_device):
  // wait limit in clock cycles (0: the default, ~1 s) and a producer that issues no loads
  int64_t split_wait_cycles = 0;
  int32_t split_withhold_loads = 0;

  // profiling
  bool profiling = false;
  std::vector<qg::KernelStat> stats;
  std::vector<qg::PendingEvent> pending;
  std::vector<cudaEvent_t> event_pool;
  int64_t launch_count = 0;
};

namespace qg {

using Ctx = qmckl_context_struct_device;

inline Ctx* ctx_of(qmckl_context_device c) { return reinterpret_cast<Ctx*>(c); }

// Error helpers (record in ctx->error like qmckl_failwith_device).
qmckl_exit_code_device fail(qmckl_context_device c, qmckl_exit_code_device code, const char* fn, const char* msg);

// Device memory owned by the context (registered, freed at destroy).
void* dalloc(Ctx* ctx, size_t bytes);
void dfree(Ctx* ctx, void* p);
// Ensures *buf holds at least `bytes`, reallocating (contents not kept) when smaller.
bool ensure(Ctx* ctx, double** buf, size_t* cap, size_t bytes);
bool ensure_raw(Ctx* ctx, void** buf, size_t* cap, size_t bytes);

// AO kernel tables (built on first use after finalize) and the processing order of the
// current points (null: identity order), both in ao_basis.cpp.
qmckl_exit_code_device ensure_tables(Ctx* ctx, qmckl_context_device c);
const int32_t* point_order(Ctx* ctx);
cudaError_t launch_exp_check(Ctx* ctx, const ExpTable* tab, const double* x, int64_t n, double* out);
cudaError_t launch_prim_check(Ctx* ctx, const AoTables& t, const double* r2, int64_t n, int64_t prim_num,
                              double* out);

// Selects the context's device and creates its stream on first use.
bool ensure_device(Ctx* ctx);
// True when a kernel may dereference p (device, managed or page-locked host memory).
bool gpu_accessible(const void* p);
// The context's grow-only staging buffer, at least `bytes` long (nullptr on failure).
void* staging(Ctx* ctx, size_t bytes);
// First recorded out-of-range store of the bounds-checked build over all translation units
// (1 found, 0 none, -1 not a bounds-checked build, -2 a CUDA error); reset clears the records.
int32_t bounds_check_status(bool reset, int64_t* site, int64_t* index, int64_t* extent);
cudaError_t bounds_selftest(int64_t index, int64_t extent);

// Synchronous unless ctx->async.
qmckl_exit_code_device finish(Ctx* ctx, qmckl_context_device c, const char* fn);
qmckl_exit_code_device copy(Ctx* ctx, qmckl_context_device c, void* dst, const void* src, size_t bytes,
                            const char* fn, bool force_sync = false);

// Kernel launch bracketing for profiling; slot names are stable strings.
struct LaunchScope {
  Ctx* ctx;
  int slot;
  cudaEvent_t start = nullptr, stop = nullptr;
  LaunchScope(Ctx* c, const char* name);
  ~LaunchScope();
};

// ---- kernel entry points (ao_kernels.cu, mo_kernels.cu, util_kernels.cu) ----
// Number of grid cells used by launch_point_order (32 per axis).
constexpr int kOrderCells = 32 * 32 * 32;
// perm <- an order of the points that puts spatial neighbours in the same warp (counting
// sort of their Morton cell keys); keys [P] and counts [kOrderCells] are scratch.
cudaError_t launch_point_order(Ctx* ctx, const AoTables& t, const double* coord, int64_t coord_ld, int64_t point_num,
                               int32_t* keys, int32_t* counts, int32_t* perm);
// The same for nr consecutive ranges of a point set of point_num points (coordinates [3][point_num]):
// range r covers points bounds[r] .. bounds[r + 1] - 1 (bounds on the device) and is ordered on its
// own; perm[bounds[r] + i] holds range-local point indices. counts holds nr * kOrderCells counters.
cudaError_t launch_point_order_ranges(Ctx* ctx, const AoTables& t, const double* coord, int64_t point_num,
                                      const int64_t* bounds, int nr, int32_t* keys, int32_t* counts, int32_t* perm);
// Fused AO kernels; perm (may be null) is the processing order of the points.
cudaError_t launch_ao_vgl(Ctx* ctx, const AoTables& t, const double* coord, const int32_t* perm, int64_t point_num,
                          double* ao_vgl);
cudaError_t launch_ao_value(Ctx* ctx, const AoTables& t, const double* coord, const int32_t* perm,
                            int64_t point_num, double* ao_value);
// AO vgl written straight as the three BF16 planes of the split-BF16 contraction, M-major:
// planes [3][kp][5 pp] with pp = point_num rounded up to 32, operand row c * pp + s holding
// component c of the point at processing slot s (perm order); AOs [ao_num, kp) are zero and
// the reference's zero-value skip is applied.
cudaError_t launch_ao_planes(Ctx* ctx, const AoTables& t, const double* coord, int64_t coord_ld, const int32_t* perm,
                             int64_t point_num, int64_t kp, void* planes);
cudaError_t launch_shell_vgl(Ctx* ctx, const AoTables& t, const double* coord, int64_t point_num,
                             int64_t shell_num, double* shell_vgl);
// mo_vgl[5P][M] = ao_vgl[5P][A] * coef_t[A][M], skipping (for components 1..4) the AOs whose
// value is exactly zero, as the reference does (src/qmckl_mo_sycl.cpp:40).
cudaError_t launch_mo_vgl_fp64(Ctx* ctx, const double* ao_vgl, const double* coef_t, int64_t point_num,
                               int64_t ao_num, int64_t mo_num, double* mo_vgl);
cudaError_t launch_mo_value_fp64(Ctx* ctx, const double* ao_value, const double* coef_t, int64_t point_num,
                                 int64_t ao_num, int64_t mo_num, double* mo_value);
cudaError_t launch_transpose(Ctx* ctx, const double* in, int64_t rows, int64_t cols, double* out);
// Plain row-major FP64 products on the DMMA pipe: C[R][N] = A[R][K] * B[K][N]; the split-K form
// sums nparts K-slices (parts: nparts x R x N scratch) in a fixed order.
cudaError_t launch_dgemm_rm(Ctx* ctx, const double* A, const double* B, double* C, int64_t R, int64_t K, int64_t N,
                            const char* name);
int64_t dgemm_splitk_parts(int64_t R, int64_t K, int64_t N, int sms);
cudaError_t launch_dgemm_splitk(Ctx* ctx, const double* A, const double* B, double* parts, int64_t nparts, double* C,
                                int64_t R, int64_t K, int64_t N, const char* name);

// ---- multi-molecule (batched) launches: one launch covers the work of every molecule ----
// Arguments of the fused AO kernel for one molecule (one warp task = 32 points x one
// nucleus chunk of the selected level).
struct FusedArgs {
  const NucleusEntry* nuclei;
  const ShellEntry* shells;
  const PrimEntry* prims;
  const double* aof;
  const NucleusChunk* chunks;
  const ExpTable* exp_table;
  const PrimFold* fold;     // AoTables::fold (split-BF16 planes only)
  const PrimFold* ent;      // AoTables::ent, or null
  int ent_cap;              // AoTables::ent_cap
  const double* coord;      // [3][coord_ld]: x of point p at coord[p], y at coord[coord_ld + p], ...
  const int32_t* perm;      // processing order of the points, or null
  double* out;              // ao_vgl (FP64 output)
  void* planes;             // BF16 planes of the split-BF16 output [3][row_len][5 plane_pp], M-major,
                            // rows in 64-point blocks: row (5 g + c) 64 + j = component c of slot
                            // 64 g + j
  int64_t point_num;
  int64_t ao_num;
  int64_t row_len;          // ao_num, or the padded K of the planes
  int64_t plane_pp;         // points rounded up to a multiple of 64
  int64_t coord_ld;         // row stride of coord (point_num, or more for a slice of a larger set)
  int64_t task_num;
  int chunk_num;
  // The point groups in nseg consecutive segments, coarse to fine: segment i covers groups from
  // seg_group[i] on, split at its own chunk level (seg_chunks, seg_chunk_num[i] chunks), and its
  // tasks are numbered from seg_task[i] (seg_task[nseg] = task_num). The finer segments at the
  // end make the last tasks the warps take short.
  static constexpr int kMaxSegments = 8;
  int nseg;
  int64_t seg_task[kMaxSegments + 1];
  int64_t seg_group[kMaxSegments];
  const NucleusChunk* seg_chunks[kMaxSegments];
  int seg_chunk_num[kMaxSegments];
};
// Number of nucleus-chunk levels of the tables (level v has about 2^v chunks).
int ao_level_count(const AoTables& t);
// Whether the fused AO kernel for ao_vgl (planes false) or the BF16 planes (true) shares the
// exponentials of t: t.ent exists and either sharing was requested explicitly or the output
// is FP64.
bool ao_shared_exponentials(const AoTables& t, bool planes);
FusedArgs make_fused_args(const AoTables& t, int level, const double* coord, const int32_t* perm, int64_t point_num,
                          double* out, void* planes, int64_t row_len);
// Ends a's schedule with finer segments: from the pieces (when `pieces`) up through the levels
// finer than a's, each holding about tail_tasks tasks, at most max_segments segments in all and at
// most half of the point groups in the finer ones.
void plan_segments(FusedArgs& a, const AoTables& t, int level, int64_t tail_tasks, int max_segments,
                   bool pieces);
// Persistent AO kernel over the tasks of nmol molecules: mols[m]'s tasks are numbered from
// task_begin[m] (non-decreasing, task_begin[nmol] = total); warps take tasks from *counter
// (zeroed before the launch). planes selects the BF16-plane output; high_l must be set when
// some molecule has shells with l >= 4; ent_cap is the largest AoTables::ent_cap of the
// molecules with shared exponentials (0: none). grid <= 0: resident CTAs.
cudaError_t launch_ao_batch(cudaStream_t stream, bool planes, bool high_l, int ent_cap, const FusedArgs* mols,
                            const int64_t* task_begin, int nmol, int64_t total, unsigned long long* counter,
                            int grid);
int ao_batch_resident_ctas(bool planes, bool high_l, int ent_cap);

// Point order of nmol molecules at once: one Morton grid per molecule, counts [nmol][kOrderCells].
struct OrderDesc {
  const double* coord;  // [3][P]
  int64_t point_num;
  int64_t point_begin;  // first global point index of the molecule
  double origin[3];
  double inv_cell;
  int32_t* keys;        // [P]
  int32_t* perm;        // [P]
};
cudaError_t launch_order_batch(cudaStream_t stream, const OrderDesc* desc, const int64_t* point_begin, int nmol,
                               int64_t total_points, int32_t* counts);

// FP64 contraction of several molecules in one persistent launch; CTA tiles are taken from
// *counter (zeroed before the launch) in job order. shape: 0 = 64x64, 1 = 128x64, 2 = 64x128.
struct GemmJob {
  const double* a;  // [rows][k]
  const double* b;  // [k][cols]
  double* c;        // [rows][cols]
  int64_t rows, k, cols;
  int32_t col_tiles;
  int32_t tile_begin;
};
constexpr int kGemmShapes = 3;
void gemm_shape_tile(int shape, int* rows, int* cols);
cudaError_t launch_dgemm_batch(cudaStream_t stream, int shape, bool mask5, const GemmJob* jobs, const int32_t* tile_begin,
                               int njobs, int total_tiles, unsigned int* counter);

// Split-BF16 contraction of several molecules: host-built descriptors (opaque here).
size_t split_job_bytes();
// Writes one job (out[rows][M] from A planes [3][rows][kp] and B planes [3][M][kp]) into
// job_host with column tiles of at most n_cap (16..160) columns; returns its tile count or -1.
int split_make_job(void* job_host, const void* a_planes, int64_t rows, const void* b_planes, int64_t M, int64_t kp,
                   double* out, int tile_begin, int n_cap);
// The same from the fused AO kernel's M-major planes ([3][kp][5 pp]; see launch_ao_planes) into
// out[5 npts][M], operand row c * pp + s landing in output row 5 perm[s] + c.
int split_make_job_mn(void* job_host, const void* a_planes, int64_t pp, int64_t npts, const int32_t* perm,
                      const void* b_planes, int64_t M, int64_t kp, double* out, int tile_begin, int n_cap);
cudaError_t split_launch_jobs(cudaStream_t stream, const void* jobs, int njobs, int total_tiles, int* err);
int64_t split_k_pad(int64_t ao_num);
// mo_vgl of the split-BF16 form computed in point ranges whose results are copied to the host
// buffer while the next range computes (the cache ends up holding the full result): `chunks`
// ranges growing by `ratio`, or with chunks = 0 ranges sized by the contraction's waves.
qmckl_exit_code_device split_mo_vgl_to_host(Ctx* ctx, qmckl_context_device c, double* host_dst, int chunks,
                                            double ratio);
// The member's coefficient planes for the split-BF16 form (built once per coefficient set)
// and its AO-plane buffer for rows x kp (returns null on allocation failure).
qmckl_exit_code_device split_prepare_coef(Ctx* ctx, qmckl_context_device c, int64_t kp);
void* split_a_planes(Ctx* ctx, int64_t rows, int64_t kp);
cudaError_t launch_strided_copy(Ctx* ctx, const double* in, int64_t in_stride, double* out, int64_t out_stride,
                                int64_t rows, int64_t cols);
cudaError_t launch_fill(Ctx* ctx, double* p, int64_t n, double v);
cudaError_t launch_point_aos_to_soa(Ctx* ctx, const double* in, int64_t num, double* out);

}  // namespace qg
