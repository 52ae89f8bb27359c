// Host runtime of libdaggergb300: library state, the tile-operation C ABI,
// and the datadeps engine that turns a recorded region of tile tasks into a
// multi-stream CUDA graph.
//
// Datadeps semantics follow Dagger.spawn_datadeps (src/datadeps/queue.jl:35-63
// of Dagger.jl): tasks are recorded in submission order; each matrix argument
// is an In / Out / InOut access over its strided byte footprint (the
// reference's StridedAliasing, src/memory-spaces.jl:480); a task that writes
// waits for the last writer and every reader since of every overlapping
// footprint, a task that reads waits for the last writer
// (src/datadeps/aliasing.jl:740-776).  Independent tasks may run in parallel;
// the result equals running the tasks one by one in submission order.
//
// Lowering: every task is given a stream from a per-thread pool.  A task
// reuses the stream of its latest predecessor when that predecessor is still
// the stream's tail (the edge is then free), otherwise it takes the least
// recently used stream; each remaining cross-stream edge becomes an event
// wait.  The issue is captured into a CUDA graph, cached by a hash of the
// task list (same tasks, same pointers -> same graph), and replayed.
#include <atomic>
#include <cstring>
#include <deque>
#include <functional>
#include <map>
#include <memory>
#include <mutex>
#include <string>
#include <unordered_map>
#include <vector>

#include "dg_common.cuh"
#include "runtime.h"

// ---------------------------------------------------------------------------
// errors, device properties
// ---------------------------------------------------------------------------
static thread_local std::string t_last_error;

void dg_set_last_error(const char *file, int line, const char *msg) {
  const char *base = strrchr(file, '/');
  t_last_error = std::string(base ? base + 1 : file) + ":" + std::to_string(line) + ": " + msg;
}

int dg_num_sms() {
  static std::atomic<int> cache[64];  // zero-initialised: not looked up yet
  int dev = 0;
  cudaGetDevice(&dev);
  if (dev < 0 || dev >= 64) dev = 0;
  int v = cache[dev].load(std::memory_order_relaxed);
  if (!v) {
    cudaDeviceGetAttribute(&v, cudaDevAttrMultiProcessorCount, dev);
    v = v > 0 ? v : 1;
    cache[dev].store(v, std::memory_order_relaxed);
  }
  return v;
}

namespace dg {

static std::atomic<long long> g_launches{0};
void count_launches(long long n) { g_launches += n; }
long long launches() { return g_launches.load(); }

DeviceState &device_state() {
  static std::mutex mu;
  static std::map<int, std::unique_ptr<DeviceState>> states;
  int dev = 0;
  cudaGetDevice(&dev);
  std::lock_guard<std::mutex> g(mu);
  auto &p = states[dev];
  if (!p) p.reset(new DeviceState());
  return *p;
}

// Per-thread pools of non-blocking streams (per device and priority level):
// level 0 at the device's greatest stream priority, each further level one
// step lower down to the least, so that the CTAs of the tasks needed soonest
// are scheduled first.
std::vector<cudaStream_t> &stream_pool(int want, int level) {
  static thread_local std::map<std::pair<int, int>, std::vector<cudaStream_t>> pools;
  int dev = 0;
  cudaGetDevice(&dev);
  auto &v = pools[{dev, level}];
  while ((int)v.size() < want) {
    cudaStream_t s;
    int least = 0, greatest = 0;
    cudaDeviceGetStreamPriorityRange(&least, &greatest);
    const int prio = (level >= kPrioLevels - 1 || greatest + level > least) ? least : greatest + level;
    if (cudaStreamCreateWithPriority(&s, cudaStreamNonBlocking, prio) != cudaSuccess) break;
    v.push_back(s);
  }
  return v;
}

int DeviceState::scratch_int(int **p) {
  std::lock_guard<std::mutex> g(mu);
  if (!info_words) {
    if (cudaMalloc((void **)&info_words, sizeof(int) * kInfoWords) != cudaSuccess) {
      dg_set_last_error(__FILE__, __LINE__, "cudaMalloc of info words failed");
      return DG_ERR_NOMEM;
    }
    cudaMemset(info_words, 0, sizeof(int) * kInfoWords);
  }
  *p = info_words + (next_info++ % kInfoWords);
  return 0;
}

Workspace *DeviceState::workspace_of(cudaStream_t s) {
  std::lock_guard<std::mutex> g(mu);
  auto &w = workspaces[s];
  if (!w) w.reset(new Workspace());
  return w.get();
}

void DeviceState::release_idle_workspaces() {
  std::lock_guard<std::mutex> g(mu);
  for (auto &kv : workspaces) {
    Workspace *w = kv.second.get();
    if (!w->p || !w->use.try_lock()) continue;  // in use: keep it
    if (!w->recorded || cudaEventSynchronize(w->done) == cudaSuccess) {
      cudaFree(w->p);
      w->p = nullptr;
      w->bytes = 0;
    }
    cudaGetLastError();
    w->use.unlock();
  }
}

int WsLease::acquire(size_t bytes, cudaStream_t s, void **p) {
  *p = nullptr;
  Workspace *w = device_state().workspace_of(s);
  w->use.lock();
  auto fail = [&](const char *what) {
    cudaGetLastError();
    dg_set_last_error(__FILE__, __LINE__, what);
    w->use.unlock();
    return DG_ERR_NOMEM;
  };
  if (!w->done && cudaEventCreateWithFlags(&w->done, cudaEventDisableTiming) != cudaSuccess)
    return fail("cannot create the workspace event");
  // the work the previous lease of this stream handle queued comes first
  if (w->recorded && cudaStreamWaitEvent(s, w->done, 0) != cudaSuccess)
    return fail("cannot order the stream after the workspace's last use");
  if (w->bytes < bytes) {
    if (w->p) {
      cudaFreeAsync(w->p, s);
      w->p = nullptr;
      w->bytes = 0;
    }
    if (pool_malloc_async(&w->p, bytes, s) != cudaSuccess) {
      w->p = nullptr;
      return fail("allocation of the emulated-FP64 / LU workspace failed");
    }
    w->bytes = bytes;
  }
  w_ = w;
  s_ = s;
  *p = w->p;
  return 0;
}

WsLease::~WsLease() {
  if (!w_) return;
  w_->recorded = cudaEventRecord(w_->done, s_) == cudaSuccess;
  if (!w_->recorded) cudaGetLastError();
  w_->use.unlock();
}

// A slot: the 8 BF16 slices of up to `cap` vectors of padded length ldk,
// one 8-byte scale word per vector, then room for a square operand's
// diagonal (kept in FP64 outside the slices).
size_t oz_slot_bytes(long long ldk, long long cap) {
  size_t b = (size_t)kOzSlices * ldk * cap * 2 + (size_t)cap * 16;
  return (b + 255) & ~(size_t)255;
}
static double *slot_diag(const void *slot, long long ldk, long long cap) {
  return (double *)((char *)slot + (size_t)kOzSlices * ldk * cap * 2 + (size_t)cap * 8);
}

DeviceState::~DeviceState() {}

// ---------------------------------------------------------------------------
// strided footprints
// ---------------------------------------------------------------------------
Footprint footprint(const void *p, int rows, int cols, int ld, int elem) {
  Footprint f;
  f.base = (uintptr_t)p;
  f.rows = (int64_t)(rows > 0 ? rows : 0) * elem;
  f.cols = cols > 0 ? cols : 0;
  f.ld = (int64_t)(ld > 0 ? ld : 1) * elem;
  f.lo = f.base;
  f.hi = (f.rows == 0 || f.cols == 0) ? f.base : f.base + (f.cols - 1) * f.ld + f.rows;
  return f;
}

static bool ranges_meet(int64_t a0, int64_t a1, int64_t b0, int64_t b1) {
  return a0 < b1 && b0 < a1;
}

bool overlaps(const Footprint &a, const Footprint &b) {
  if (a.hi <= b.lo || b.hi <= a.lo) return false;
  if (a.ld != b.ld || a.rows > a.ld || b.rows > b.ld) return true;  // conservative
  const Footprint &x = a.base <= b.base ? a : b;
  const Footprint &y = a.base <= b.base ? b : a;
  int64_t d = (int64_t)(y.base - x.base);
  int64_t cb = d / x.ld, rb = d % x.ld;
  // y's rows [rb, rb + y.rows) in x's columns [cb, cb + y.cols); rows past
  // ld wrap into the next column.
  int64_t r_end = rb + y.rows;
  if (ranges_meet(0, x.rows, rb, r_end < x.ld ? r_end : x.ld) &&
      ranges_meet(0, x.cols, cb, cb + y.cols))
    return true;
  if (r_end > x.ld && ranges_meet(0, x.rows, 0, r_end - x.ld) &&
      ranges_meet(0, x.cols, cb + 1, cb + 1 + y.cols))
    return true;
  return false;
}

}  // namespace dg

// ---------------------------------------------------------------------------
// the region (datadeps engine)
// ---------------------------------------------------------------------------
using dg::Footprint;

struct dg_region {
  struct Access {
    Footprint f;
    int mode;
  };
  struct Ainfo {
    Footprint f;
    int last_writer = -1;
    std::vector<int> readers;
  };
  std::vector<dg_task> tasks;
  std::vector<char> level;  // priority level, 0 = critical path (kPrioLevels - 1 by default)
  std::vector<std::vector<int>> preds;
  std::vector<Ainfo> ainfos;
  std::multimap<uintptr_t, int> by_lo;
  uint64_t max_len = 0;
  uint64_t hash = 1469598103934665603ull;
  int nedges = 0;
  std::deque<std::vector<double *>> tables;  // tile lists of OP_LU_LASWP / OP_LU_ROWS
};

static void hash_bytes(uint64_t &h, const void *p, size_t n) {
  const unsigned char *c = (const unsigned char *)p;
  for (size_t i = 0; i < n; i++) {
    h ^= c[i];
    h *= 1099511628211ull;
  }
}

static void task_accesses(const dg_task &t, std::vector<dg_region::Access> &out) {
  out.clear();
  auto mode = [](int m, int def) { return m ? m : def; };
  const int E = 8;
  switch (t.op) {
    case DG_OP_POTRF:
    case dg::OP_OZ_POTRF:
      out.push_back({dg::footprint(t.c, t.n, t.n, t.ldc, E), mode(t.mode_c, DG_INOUT)});
      if (t.op == dg::OP_OZ_POTRF)
        out.push_back({dg::footprint(t.b, t.ldb, 1, 1, 256), DG_OUT});  // slice scratch
      break;
    case dg::OP_OZ_ZERO:
      out.push_back({dg::footprint(t.c, t.m, t.n, t.ldc, E), DG_OUT});
      break;
    case dg::OP_TILE_T:
      out.push_back({dg::footprint(t.a, t.m, t.n, t.lda, E), DG_IN});
      out.push_back({dg::footprint(t.c, t.n, t.m, t.ldc, E), DG_OUT});
      break;
    case dg::OP_TILE_MIRROR:
      out.push_back({dg::footprint(t.c, t.n, t.n, t.ldc, E), DG_INOUT});
      break;
    case dg::OP_UPLOAD:  // the source is row-major: n contiguous values per row
      out.push_back({dg::footprint(t.a, t.n, t.m, t.lda, E), DG_IN});
      out.push_back({dg::footprint(t.c, t.m, t.n, t.ldc, E), DG_OUT});
      break;
    case dg::OP_OZ_INV:
      out.push_back({dg::footprint(t.a, t.n, t.n, t.lda, E), DG_IN});
      out.push_back({dg::footprint(t.c, t.n, t.n, t.ldc, E), DG_OUT});
      out.push_back({dg::footprint(t.b, t.ldb, 1, 1, 256), DG_OUT});  // slice scratch
      break;
    case DG_OP_TRSM:
    case dg::OP_OZ_TRSM: {
      int ka = (t.side == 'L' || t.side == 'l') ? t.m : t.n;
      out.push_back({dg::footprint(t.a, ka, ka, t.lda, E), mode(t.mode_a, DG_IN)});
      out.push_back({dg::footprint(t.c, t.m, t.n, t.ldc, E), mode(t.mode_c, DG_INOUT)});
      if (t.op == dg::OP_OZ_TRSM)
        out.push_back({dg::footprint(t.b, t.ldb, 1, 1, 256), DG_OUT});  // slice scratch
      break;
    }
    case DG_OP_SYRK: {
      bool nt = (t.trans == 'N' || t.trans == 'n');
      out.push_back({dg::footprint(t.a, nt ? t.n : t.k, nt ? t.k : t.n, t.lda, E), mode(t.mode_a, DG_IN)});
      out.push_back({dg::footprint(t.c, t.n, t.n, t.ldc, E), mode(t.mode_c, DG_INOUT)});
      break;
    }
    case DG_OP_GEMM: {
      bool na = (t.transa == 'N' || t.transa == 'n'), nb = (t.transb == 'N' || t.transb == 'n');
      out.push_back({dg::footprint(t.a, na ? t.m : t.k, na ? t.k : t.m, t.lda, E), mode(t.mode_a, DG_IN)});
      out.push_back({dg::footprint(t.b, nb ? t.k : t.n, nb ? t.n : t.k, t.ldb, E), mode(t.mode_b, DG_IN)});
      out.push_back({dg::footprint(t.c, t.m, t.n, t.ldc, E), mode(t.mode_c, t.beta == 0.0 ? DG_OUT : DG_INOUT)});
      break;
    }
    case DG_OP_COPY:
      out.push_back({dg::footprint(t.a, t.m, t.n, t.lda, E), mode(t.mode_a, DG_IN)});
      out.push_back({dg::footprint(t.c, t.m, t.n, t.ldc, E), mode(t.mode_c, DG_OUT)});
      break;
    case dg::OP_OZ_SPLIT: {
      const bool cols = (t.trans == 'N');
      out.push_back({dg::footprint(t.a, cols ? t.m : t.n, cols ? t.n : t.m, t.lda, E), DG_IN});
      out.push_back({dg::footprint(t.c, (int)dg::oz_slot_bytes(t.ldc, t.k), 1, 1, 1), DG_OUT});
      break;
    }
    case dg::OP_OZ_GEMM:
      out.push_back({dg::footprint(t.a, (int)dg::oz_slot_bytes(t.lda, t.ldb), 1, 1, 1), DG_IN});
      out.push_back({dg::footprint(t.b, (int)dg::oz_slot_bytes(t.lda, t.ldb), 1, 1, 1), DG_IN});
      out.push_back({dg::footprint(t.c, t.m, t.n, t.ldc, E), DG_INOUT});
      break;
    case dg::OP_LU_PANEL: {
      out.push_back({dg::footprint(t.c, t.m, t.n, t.ldc, E), DG_INOUT});
      const bool piv = (t.transa == 'P');
      const dg::LuLayout L = dg::lu_layout(t.lda, t.k, t.ldb, piv, t.diag == 'E');
      const char *ws = (const char *)t.b;
      const int step = t.info_offset / t.ldb;
      // the leaf scratch and the panel's emulated-update scratch
      out.push_back({dg::footprint(ws + L.leaf, (int)(L.lpiv - L.leaf), 1, 1, 1), DG_OUT});
      if (L.ozp_bytes)
        out.push_back({dg::footprint(ws + L.ozp, (int)(L.ozp_bytes / 256), 1, 1, 256), DG_OUT});
      // this step's slice of the leaves' pivot rows (panel rows per column)
      const int npanel = t.m < t.n ? t.m : t.n;
      if (npanel > 0)
        out.push_back({dg::footprint(ws + L.lpiv + (size_t)t.info_offset * 4, npanel, 1, 1, 4),
                       DG_OUT});
      // The info word (an atomicMin of the first zero pivot's column) and the
      // status word (a sticky error code) take no edge: every step only
      // lowers or sets them and nothing inside the region reads them for
      // ordering; the host reads both after the region.
      if (piv) {
        const int npiv = t.m < t.n ? t.m : t.n;
        out.push_back({dg::footprint(ws + L.lists + (size_t)step * L.list_stride * 4,
                                     (int)L.list_stride, 1, 1, 4), DG_OUT});
        out.push_back({dg::footprint((const long long *)t.a + t.info_offset, npiv, 1, 1, 8),
                       DG_OUT});
      }
      break;
    }
    case dg::OP_LU_LASWP:
    case dg::OP_LU_ROWS: {
      double *const *tl = (double *const *)t.a;
      for (int i = 0; i < t.k; i++) {
        const int rows = (i == t.k - 1) ? t.m - i * t.ldb : t.ldb;
        out.push_back({dg::footprint(tl[i], rows, t.n, rows, E), DG_INOUT});
      }
      if (t.op == dg::OP_LU_LASWP) {
        out.push_back({dg::footprint(t.b, 1 + 2 * t.ldc, 1, 1, 4), DG_IN});
      } else {
        out.push_back({dg::footprint(t.b, t.m, 1, 1, 4), DG_IN});
        out.push_back({dg::footprint(t.c, t.m, t.n, t.m, E), DG_OUT});
      }
      break;
    }
    case dg::OP_LU_LINV:
      out.push_back({dg::footprint(t.a, t.n, t.n, t.lda, E), DG_IN});
      out.push_back({dg::footprint(t.c, t.n, t.n, t.ldc, E), DG_OUT});
      break;
    case dg::OP_LU_PERM:
      out.push_back({dg::footprint(t.a, t.k, 1, 1, 8), DG_IN});
      out.push_back({dg::footprint(t.c, t.n, 1, 1, 4), DG_OUT});
      break;
  }
}

extern "C" dg_region *dg_region_create(void) { return new dg_region(); }
extern "C" void dg_region_destroy(dg_region *r) { delete r; }

extern "C" int dg_region_add(dg_region *r, const dg_task *tp) {
  DG_CHECK_ARG(r != nullptr, 1);
  DG_CHECK_ARG(tp != nullptr, 2);
  const dg_task &t = *tp;
  DG_CHECK_ARG((t.op >= DG_OP_POTRF && t.op <= DG_OP_COPY) ||
                   (t.op >= dg::OP_OZ_SPLIT && t.op <= dg::kOpLast),
               2);
  const int id = (int)r->tasks.size();
  r->tasks.push_back(t);
  r->level.push_back((char)(dg::kPrioLevels - 1));
  hash_bytes(r->hash, &t, sizeof(dg_task));
  if (t.op == dg::OP_LU_LASWP || t.op == dg::OP_LU_ROWS)  // the tiles, not the list's address
    hash_bytes(r->hash, t.a, sizeof(double *) * (size_t)t.k);
  std::vector<dg_region::Access> acc;
  task_accesses(t, acc);
  std::vector<int> p;
  auto add = [&](int q) {
    if (q < 0 || q == id) return;
    for (int x : p)
      if (x == q) return;
    p.push_back(q);
  };
  std::vector<int> exact(acc.size(), -1);
  for (size_t ai = 0; ai < acc.size(); ai++) {
    const Footprint &f = acc[ai].f;
    if (f.hi == f.lo) continue;
    uintptr_t from = f.lo > r->max_len ? f.lo - r->max_len : 0;
    for (auto it = r->by_lo.lower_bound(from); it != r->by_lo.end() && it->first < f.hi; ++it) {
      dg_region::Ainfo &o = r->ainfos[it->second];
      if (!dg::overlaps(o.f, f)) continue;
      if (o.f.base == f.base && o.f.rows == f.rows && o.f.cols == f.cols && o.f.ld == f.ld)
        exact[ai] = it->second;
      add(o.last_writer);                       // both reads and writes
      if (acc[ai].mode & DG_OUT)
        for (int q : o.readers) add(q);         // writes also wait for readers
    }
  }
  for (size_t ai = 0; ai < acc.size(); ai++) {
    const Footprint &f = acc[ai].f;
    if (f.hi == f.lo) continue;
    int idx = exact[ai];
    if (idx < 0) {
      idx = (int)r->ainfos.size();
      r->ainfos.push_back({f, -1, {}});
      r->by_lo.emplace(f.lo, idx);
      if (f.hi - f.lo > r->max_len) r->max_len = f.hi - f.lo;
      exact[ai] = idx;
    }
    dg_region::Ainfo &o = r->ainfos[idx];
    if (acc[ai].mode & DG_OUT) {
      o.last_writer = id;
      o.readers.clear();
    } else {
      o.readers.push_back(id);
    }
  }
  // an access both read and written by this task (InOut) ends as a write
  for (size_t ai = 0; ai < acc.size(); ai++) {
    if (exact[ai] < 0) continue;
    dg_region::Ainfo &o = r->ainfos[exact[ai]];
    if (o.last_writer == id) {
      std::vector<int> keep;
      for (int q : o.readers)
        if (q != id) keep.push_back(q);
      o.readers.swap(keep);
    }
  }
  r->nedges += (int)p.size();
  r->preds.push_back(std::move(p));
  return 0;
}

extern "C" int dg_region_stats(const dg_region *r, int *ntasks, int *nedges) {
  DG_CHECK_ARG(r != nullptr, 1);
  if (ntasks) *ntasks = (int)r->tasks.size();
  if (nedges) *nedges = r->nedges;
  return 0;
}

extern "C" int dg_region_edges(const dg_region *r, int *pairs, int cap) {
  DG_CHECK_ARG(r != nullptr, 1);
  int n = 0;
  for (size_t t = 0; t < r->preds.size(); t++)
    for (int q : r->preds[t]) {
      if (n >= cap) return n;
      pairs[2 * n] = (int)t;
      pairs[2 * n + 1] = q;
      n++;
    }
  return n;
}

namespace dg {

int run_task(const dg_task &t, int *info, cudaStream_t s) {
  switch (t.op) {
    case DG_OP_POTRF:
      return potrf_f64(t.uplo, t.n, t.c, t.ldc, info, t.info_offset, s);
    case DG_OP_TRSM:
      return trsm_f64(t.side, t.uplo, t.transa, t.diag, t.m, t.n, t.alpha, t.a, t.lda, t.c, t.ldc,
                      info, s);
    case OP_OZ_POTRF:
      return potrf_f64_oz(t.uplo, t.n, t.c, t.ldc, info, t.info_offset, (void *)t.b,
                          (size_t)t.ldb * 256, s);
    case OP_UPLOAD:
      return upload_tile(t.a, t.lda, t.m, t.n, t.c, s);
    case OP_TILE_T:
      return tile_transpose(t.a, t.lda, t.m, t.n, t.c, t.ldc, s);
    case OP_TILE_MIRROR:
      return tile_mirror_upper(t.c, t.ldc, t.n, s);
    case OP_OZ_ZERO:
      if (t.m <= 0 || t.n <= 0) return 0;
      DG_CUDA_TRY(cudaMemset2DAsync(t.c, (size_t)t.ldc * 8, 0, (size_t)t.m * 8, t.n, s));
      return 0;
    case OP_OZ_INV:  // W = U^-T (upper) or L^-T (lower), one column per CTA
      return trinv_t_f64(t.uplo, t.n, t.a, t.lda, t.c, t.ldc, info, s);
    case OP_OZ_TRSM:
      return trsm_f64_oz(t.side, t.uplo, t.transa, t.diag, t.m, t.n, t.alpha, t.a, t.lda, t.c,
                         t.ldc, (void *)t.b, (size_t)t.ldb * 256, info, s);
    case DG_OP_SYRK: {
      bool nt = (t.trans == 'N' || t.trans == 'n');
      Tri tri = (t.uplo == 'U' || t.uplo == 'u') ? TRI_UPPER : TRI_LOWER;
      return gemm_f64(nt ? 'N' : 'T', nt ? 'T' : 'N', t.n, t.n, t.k, t.alpha, t.a, t.lda, t.a,
                      t.lda, t.beta, t.c, t.ldc, tri, info, s);
    }
    case DG_OP_GEMM:
      return gemm_f64(t.transa, t.transb, t.m, t.n, t.k, t.alpha, t.a, t.lda, t.b, t.ldb, t.beta,
                      t.c, t.ldc, TRI_NONE, info, s);
    case OP_OZ_SPLIT: {
      const bool cols = (t.trans == 'N');
      const long long sstride = (long long)t.ldc * t.k;
      auto *e = (unsigned long long *)((char *)t.c + (size_t)kOzSlices * sstride * 2);
      // diag 'Z': the diagonal is kept apart in FP64 (the inverse of a triangle)
      double *dg = (t.diag == 'Z') ? slot_diag(t.c, t.ldc, t.k) : nullptr;
      return oz_split(t.a, cols ? t.lda : 1, cols ? 1 : t.lda, t.m, t.n, t.c, t.ldc, sstride, e,
                      info, s, nullptr, dg);
    }
    case OP_OZ_GEMM: {
      const long long sstride = (long long)t.lda * t.ldb;
      auto *ea = (const unsigned long long *)((const char *)t.a + (size_t)kOzSlices * sstride * 2);
      auto *eb = (const unsigned long long *)((const char *)t.b + (size_t)kOzSlices * sstride * 2);
      const int tri = (t.uplo == 'U' || t.uplo == 'u') ? 1 : (t.uplo == 'L' || t.uplo == 'l') ? 2 : 0;
      // side 'A' / 'B': the A (rows) / B (columns) operand's FP64 diagonal scales C
      const double *ds = (t.side == 'A') ? slot_diag(t.a, t.lda, t.ldb)
                         : (t.side == 'B') ? slot_diag(t.b, t.lda, t.ldb) : nullptr;
      return oz_gemm(t.m, t.n, t.k, t.alpha, t.a, t.lda, sstride, ea, t.b, t.lda, sstride, eb,
                     t.beta, t.c, t.ldc, tri, info, s, nullptr, ds, t.side == 'A' ? 1 : 2,
                     t.diag == 'P' ? kOzBlocksPerCta
                     : (t.diag >= '2' && t.diag <= '9') ? t.diag - '0' : 1);
    }
    case DG_OP_COPY:
      if (t.m <= 0 || t.n <= 0) return 0;
      DG_CUDA_TRY(cudaMemcpy2DAsync(t.c, (size_t)t.ldc * 8, t.a, (size_t)t.lda * 8, (size_t)t.m * 8,
                                    t.n, cudaMemcpyDeviceToDevice, s));
      return 0;
    case OP_LU_PANEL: {
      const bool piv = (t.transa == 'P');
      const LuLayout L = lu_layout(t.lda, t.k, t.ldb, piv, t.diag == 'E');
      char *ws = (char *)t.b;
      const int step = t.info_offset / t.ldb;
      return lu_panel_f64(t.c, t.ldc, t.m, t.n, piv, (int *)(ws + L.lpiv) + t.info_offset,
                          (int *)(ws + L.info), t.info_offset, ws + L.leaf, (int *)(ws + L.status),
                          L.ozp_bytes ? ws + L.ozp : nullptr, L.ozp_bytes,
                          (long long *)t.a + t.info_offset,
                          (int *)(ws + L.lists) + (size_t)step * L.list_stride, L.list_cap, s);
    }
    case OP_LU_LASWP:
      return lu_laswp_tiles((double *const *)t.a, t.k, t.ldb, t.m, t.n, (const int *)t.b, t.ldc, s);
    case OP_LU_PERM:
      return lu_perm((const long long *)t.a, t.k, t.n, (int *)t.c, s);
    case OP_LU_LINV:
      return trinv_unit_lower_f64(t.n, t.a, t.lda, t.c, t.ldc, info, s);
    case OP_LU_ROWS:
      return lu_rows_tiles((double *const *)t.a, t.k, t.ldb, t.m, t.n, (const int *)t.b, t.c, s);
  }
  return DG_ERR_UNSUPPORTED;
}

struct Plan {
  std::vector<int> stream_of;
  std::vector<char> needs_event;
  int nstreams = 0;
  std::vector<std::pair<int, int>> classes;  // (priority level, streams), in stream order
};

// One class of streams per priority level in use: kUrgentStreams streams for
// each level above the lowest (at most half the pool), `pool` for the lowest.  Within its class a
// task reuses the stream of its latest predecessor when that predecessor is
// still the stream's tail, else the least recently used stream.
static Plan plan_streams(const dg_region &r, int pool) {
  Plan pl;
  const int n = (int)r.tasks.size();
  std::vector<int> first(kPrioLevels + 1, -1), count(kPrioLevels + 1, 0);
  std::vector<char> used(kPrioLevels + 1, 0);
  for (int t = 0; t < n; t++) used[r.level[t]] = 1;
  int total = 0;
  for (int l = 0; l <= kPrioLevels; l++) {
    if (!used[l]) continue;
    first[l] = total;
    count[l] = (l == kTransferLevel) ? kTransferStreams
               : (l == kPrioLevels - 1) ? pool : std::min(kUrgentStreams, std::max(1, pool / 2));
    total += count[l];
    pl.classes.push_back({l, count[l]});
  }
  pl.stream_of.assign(n, 0);
  pl.needs_event.assign(n, 0);
  std::vector<int> tail(total, -1);
  std::vector<long> last_use(total, -1);
  for (int t = 0; t < n; t++) {
    const int s0 = first[r.level[t]], s1 = s0 + count[r.level[t]];
    int best = -1, bestp = -1;
    for (int q : r.preds[t]) {
      int s = pl.stream_of[q];
      if (s >= s0 && s < s1 && tail[s] == q && q > bestp) { best = s; bestp = q; }
    }
    if (best < 0) {
      best = s0;
      for (int s = s0 + 1; s < s1; s++)
        if (last_use[s] < last_use[best]) best = s;
    }
    pl.stream_of[t] = best;
    tail[best] = t;
    last_use[best] = t;
    for (int q : r.preds[t])
      if (pl.stream_of[q] != best) pl.needs_event[q] = 1;
  }
  pl.nstreams = total;
  return pl;
}

void mark_level(dg_region *r, int level) {
  if (r->level.empty()) return;
  level = level < 0 ? 0 : level > kPrioLevels - 1 ? kPrioLevels - 1 : level;
  r->level.back() = (char)level;
  const int id = (int)r->level.size() - 1;
  hash_bytes(r->hash, &id, sizeof id);
  hash_bytes(r->hash, &level, sizeof level);
}

void mark_urgent(dg_region *r) { mark_level(r, 0); }

void mark_transfer(dg_region *r) {
  if (r->level.empty()) return;
  r->level.back() = (char)kTransferLevel;
  const int id = (int)r->level.size() - 1;
  hash_bytes(r->hash, &id, sizeof id);
  hash_bytes(r->hash, &kTransferLevel, sizeof kTransferLevel);
}

// An executable graph and its info word, shared by the cache and every
// launch being issued: an eviction or a clear on one thread never destroys a
// graph that another thread is about to launch (the last holder destroys it;
// a graph still running on the device finishes first).
struct GraphObj {
  cudaGraphExec_t exec = nullptr;
  int *info = nullptr;
  long long nodes = 0;  // kernel launches captured in the graph
  GraphObj() = default;
  GraphObj(const GraphObj &) = delete;
  GraphObj &operator=(const GraphObj &) = delete;
  ~GraphObj() {
    if (exec) cudaGraphExecDestroy(exec);
    if (info) cudaFree(info);
  }
};

struct GraphEntry {
  std::shared_ptr<GraphObj> g;
  uint64_t last_used = 0;
};

static std::mutex g_graph_mu;
static std::map<std::pair<int, uint64_t>, GraphEntry> g_graphs;
static uint64_t g_graph_clock = 0;
static const size_t kMaxGraphs = 32;

static int issue(const dg_region &r, const Plan &pl, int *info, cudaStream_t origin, bool serial,
                 std::vector<cudaEvent_t> &events) {
  DG_CUDA_TRY(cudaMemsetAsync(info, 0, sizeof(int), origin));
  const int n = (int)r.tasks.size();
  if (serial) {
    for (int t = 0; t < n; t++) {
      int rc = run_task(r.tasks[t], info, origin);
      if (rc) return rc;
    }
    return 0;
  }
  std::vector<cudaStream_t> pool;
  for (const auto &c : pl.classes) {
    auto &v = stream_pool(c.second, c.first);
    if ((int)v.size() < c.second) return DG_ERR_CUDA;
    pool.insert(pool.end(), v.begin(), v.begin() + c.second);
  }
  cudaEvent_t fork;
  DG_CUDA_TRY(cudaEventCreateWithFlags(&fork, cudaEventDisableTiming));
  events.push_back(fork);
  DG_CUDA_TRY(cudaEventRecord(fork, origin));
  for (int s = 0; s < pl.nstreams; s++) DG_CUDA_TRY(cudaStreamWaitEvent(pool[s], fork, 0));
  std::vector<cudaEvent_t> ev(n, nullptr);
  for (int t = 0; t < n; t++) {
    cudaStream_t s = pool[pl.stream_of[t]];
    for (int q : r.preds[t])
      if (pl.stream_of[q] != pl.stream_of[t]) DG_CUDA_TRY(cudaStreamWaitEvent(s, ev[q], 0));
    int rc = run_task(r.tasks[t], info, s);
    if (rc) return rc;
    if (pl.needs_event[t]) {
      DG_CUDA_TRY(cudaEventCreateWithFlags(&ev[t], cudaEventDisableTiming));
      events.push_back(ev[t]);
      DG_CUDA_TRY(cudaEventRecord(ev[t], s));
    }
  }
  for (int s = 0; s < pl.nstreams; s++) {
    cudaEvent_t j;
    DG_CUDA_TRY(cudaEventCreateWithFlags(&j, cudaEventDisableTiming));
    events.push_back(j);
    DG_CUDA_TRY(cudaEventRecord(j, pool[s]));
    DG_CUDA_TRY(cudaStreamWaitEvent(origin, j, 0));
  }
  return 0;
}

static int read_info(int *info, cudaStream_t s) {
  int h = 0;
  DG_CUDA_TRY(cudaMemcpyAsync(&h, info, sizeof(int), cudaMemcpyDeviceToHost, s));
  DG_CUDA_TRY(cudaStreamSynchronize(s));
  return h;
}

// A private non-blocking stream per (thread, device): graphs cannot be
// captured on the legacy default stream, so a region handed the default
// stream is captured and launched here, bridged to the caller's stream by
// events on both sides.
static cudaStream_t private_stream() {
  static thread_local std::map<int, cudaStream_t> ps;
  int dev = 0;
  cudaGetDevice(&dev);
  auto it = ps.find(dev);
  if (it != ps.end()) return it->second;
  cudaStream_t s = nullptr;
  cudaStreamCreateWithFlags(&s, cudaStreamNonBlocking);
  ps[dev] = s;
  return s;
}

static int region_run_on(dg_region *r, int use_graph, int serial, cudaStream_t origin,
                         int stream_pool_size, bool sync);

int region_run(dg_region *r, int use_graph, int serial, cudaStream_t origin, int stream_pool_size,
               bool sync) {
  const bool legacy = origin == nullptr || origin == cudaStreamLegacy || origin == cudaStreamPerThread;
  if (!use_graph || !legacy) return region_run_on(r, use_graph, serial, origin, stream_pool_size, sync);
  cudaStream_t ps = private_stream();
  if (!ps) {
    dg_set_last_error(__FILE__, __LINE__, "cannot create a capture stream");
    return DG_ERR_CUDA;
  }
  cudaEvent_t in, out;
  DG_CUDA_TRY(cudaEventCreateWithFlags(&in, cudaEventDisableTiming));
  DG_CUDA_TRY(cudaEventCreateWithFlags(&out, cudaEventDisableTiming));
  DG_CUDA_TRY(cudaEventRecord(in, origin));
  DG_CUDA_TRY(cudaStreamWaitEvent(ps, in, 0));
  int rc = region_run_on(r, use_graph, serial, ps, stream_pool_size, sync);
  cudaEventRecord(out, ps);
  cudaStreamWaitEvent(origin, out, 0);
  cudaEventDestroy(in);
  cudaEventDestroy(out);
  return rc;
}

static int region_run_on(dg_region *r, int use_graph, int serial, cudaStream_t origin,
                         int stream_pool_size, bool sync) {
  const int n = (int)r->tasks.size();
  if (n == 0) return 0;
  Plan pl;
  if (!serial) pl = plan_streams(*r, stream_pool_size);
  std::vector<cudaEvent_t> events;
  auto cleanup = [&]() {
    for (auto e : events) cudaEventDestroy(e);
  };
  if (!use_graph) {
    int *info = nullptr;
    int rc = device_state().scratch_int(&info);
    if (rc) return rc;
    rc = issue(*r, pl, info, origin, serial, events);
    cleanup();
    if (rc) return rc;
    return sync ? read_info(info, origin) : 0;
  }
  int dev = 0;
  cudaGetDevice(&dev);
  uint64_t key = r->hash ^ ((uint64_t)serial << 63) ^ ((uint64_t)stream_pool_size << 40);
  std::shared_ptr<GraphObj> entry;
  {
    std::lock_guard<std::mutex> g(g_graph_mu);
    auto it = g_graphs.find({dev, key});
    if (it != g_graphs.end()) {
      it->second.last_used = ++g_graph_clock;
      entry = it->second.g;
    }
  }
  if (!entry) {
    entry = std::make_shared<GraphObj>();
    DG_CUDA_TRY(cudaMalloc((void **)&entry->info, 256));
    DG_CUDA_TRY(cudaMemset(entry->info, 0, 256));
    cudaGraph_t graph;
    DG_CUDA_TRY(cudaStreamBeginCapture(origin, cudaStreamCaptureModeThreadLocal));
    const long long before = launches();
    int rc = issue(*r, pl, entry->info, origin, serial, events);
    entry->nodes = launches() - before;
    count_launches(-entry->nodes);  // captured, not executed
    cudaError_t e = cudaStreamEndCapture(origin, &graph);
    cleanup();
    if (rc) {
      if (e == cudaSuccess) cudaGraphDestroy(graph);
      return rc;
    }
    DG_CUDA_TRY(e);
    // kernel nodes keep the priority of the stream they were captured from
    e = cudaGraphInstantiateWithFlags(&entry->exec, graph, cudaGraphInstantiateFlagUseNodePriority);
    cudaGraphDestroy(graph);
    if (e != cudaSuccess) {
      // A region too large for an executable graph (its nodes' memory) runs
      // on the same streams and events without one: the same tasks, order
      // and results, with the host issuing every launch.
      cudaGetLastError();
      entry->exec = nullptr;
      entry.reset();
      int *info = nullptr;
      rc = device_state().scratch_int(&info);
      if (rc) return rc;
      std::vector<cudaEvent_t> ev2;
      rc = issue(*r, pl, info, origin, serial, ev2);
      for (auto x : ev2) cudaEventDestroy(x);
      if (rc) return rc;
      return sync ? read_info(info, origin) : 0;
    }
    std::shared_ptr<GraphObj> evicted;  // destroyed after the lock is released
    {
      std::lock_guard<std::mutex> g(g_graph_mu);
      if (g_graphs.size() >= kMaxGraphs) {
        auto victim = g_graphs.begin();
        for (auto it = g_graphs.begin(); it != g_graphs.end(); ++it)
          if (it->second.last_used < victim->second.last_used) victim = it;
        evicted = std::move(victim->second.g);
        g_graphs.erase(victim);
      }
      GraphEntry ge;
      ge.g = entry;
      ge.last_used = ++g_graph_clock;
      g_graphs[{dev, key}] = ge;
    }
  }
  DG_CUDA_TRY(cudaGraphLaunch(entry->exec, origin));
  count_launches(entry->nodes);
  return sync ? read_info(entry->info, origin) : 0;
}

// Launches the cached graph of `key` on origin (a legacy stream bridged to
// the private capture stream as region_run does); false when it is not cached
// (never built, evicted or cleared).
static bool launch_cached(uint64_t key, cudaStream_t origin, bool sync, int *rc) {
  int dev = 0;
  cudaGetDevice(&dev);
  std::shared_ptr<GraphObj> entry;
  {
    std::lock_guard<std::mutex> g(g_graph_mu);
    auto it = g_graphs.find({dev, key});
    if (it == g_graphs.end()) return false;
    it->second.last_used = ++g_graph_clock;
    entry = it->second.g;
  }
  const bool legacy = origin == nullptr || origin == cudaStreamLegacy || origin == cudaStreamPerThread;
  cudaStream_t s = origin;
  cudaEvent_t in = nullptr, out = nullptr;
  if (legacy) {
    s = private_stream();
    if (!s || cudaEventCreateWithFlags(&in, cudaEventDisableTiming) != cudaSuccess ||
        cudaEventCreateWithFlags(&out, cudaEventDisableTiming) != cudaSuccess) {
      cudaGetLastError();
      if (in) cudaEventDestroy(in);
      return false;
    }
    cudaEventRecord(in, origin);
    cudaStreamWaitEvent(s, in, 0);
  }
  *rc = 0;
  if (cudaGraphLaunch(entry->exec, s) != cudaSuccess) {
    cudaGetLastError();
    dg_set_last_error(__FILE__, __LINE__, "cudaGraphLaunch failed");
    *rc = DG_ERR_CUDA;
  } else {
    count_launches(entry->nodes);
  }
  if (legacy) {
    cudaEventRecord(out, s);
    cudaStreamWaitEvent(origin, out, 0);
    cudaEventDestroy(in);
    cudaEventDestroy(out);
  }
  if (*rc == 0 && sync) *rc = read_info(entry->info, s);
  return true;
}

// Whole-call cache: the hashed arguments of a region-building entry point ->
// the key of its graph, so that a repeated call (same tiles, sizes, engine,
// workspace) launches the graph without rebuilding the region and its stream
// plan (about 8 ms of host time for the 7 k tasks of N = 32768, during which
// the GPU would idle).
static std::mutex g_call_mu;
static std::unordered_map<uint64_t, uint64_t> g_calls;

int region_run_cached(uint64_t call, const std::function<void(dg_region *)> &build,
                      cudaStream_t origin, bool sync, int streams) {
  int dev = 0;
  cudaGetDevice(&dev);
  const int engine = get_f64_engine();
  hash_bytes(call, &dev, sizeof dev);
  hash_bytes(call, &engine, sizeof engine);
  hash_bytes(call, &streams, sizeof streams);
  uint64_t key = 0;
  bool known = false;
  {
    std::lock_guard<std::mutex> g(g_call_mu);
    auto it = g_calls.find(call);
    if (it != g_calls.end()) {
      key = it->second;
      known = true;
    }
  }
  int rc = 0;
  if (known && launch_cached(key, origin, sync, &rc)) return rc;
  dg_region r;
  build(&r);
  rc = region_run(&r, 1, 0, origin, streams, sync);
  if (rc >= 0) {
    std::lock_guard<std::mutex> g(g_call_mu);
    if (g_calls.size() > 4096) g_calls.clear();
    g_calls[call] = r.hash ^ ((uint64_t)streams << 40);
  }
  return rc;
}

// The hash of a call's arguments (region_run_cached).
uint64_t call_hash(int fn, const void *args, size_t bytes, const void *const *ptrs, size_t nptrs) {
  uint64_t h = 1469598103934665603ull;
  hash_bytes(h, &fn, sizeof fn);
  hash_bytes(h, args, bytes);
  if (nptrs) hash_bytes(h, ptrs, nptrs * sizeof(void *));
  return h;
}

void clear_graphs() {
  std::vector<std::shared_ptr<GraphObj>> dropped;  // destroyed after the lock is released
  std::lock_guard<std::mutex> g(g_graph_mu);
  int dev = 0;
  cudaGetDevice(&dev);
  for (auto it = g_graphs.begin(); it != g_graphs.end();) {
    if (it->first.first == dev) {
      dropped.push_back(std::move(it->second.g));
      it = g_graphs.erase(it);
    } else {
      ++it;
    }
  }
}

}  // namespace dg

extern "C" int dg_region_run(dg_region *r, int use_graph, int serial, void *stream) {
  DG_CHECK_ARG(r != nullptr, 1);
  return dg::region_run(r, use_graph, serial, (cudaStream_t)stream, dg::kDefaultStreams, true);
}

// ---------------------------------------------------------------------------
// tile-operation ABI
// ---------------------------------------------------------------------------
static bool is_one_of(char c, const char *set) { return c && strchr(set, c) != nullptr; }

extern "C" const char *dg_version(void) { return "libdaggergb300 0.1 (sm_103a)"; }
extern "C" const char *dg_last_error(void) { return t_last_error.c_str(); }

namespace dg {
namespace {
std::mutex g_pool_mu;
cudaMemPool_t g_pools[64] = {};
}  // namespace

cudaError_t pool_malloc_async(void **p, size_t bytes, cudaStream_t s) {
  int dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) return e;
  if (dev < 0 || dev >= 64) return cudaMallocAsync(p, bytes, s);
  cudaMemPool_t pool;
  {
    std::lock_guard<std::mutex> g(g_pool_mu);
    if (!g_pools[dev]) {
      cudaMemPoolProps props;
      memset(&props, 0, sizeof props);
      props.allocType = cudaMemAllocationTypePinned;
      props.location.type = cudaMemLocationTypeDevice;
      props.location.id = dev;
      e = cudaMemPoolCreate(&g_pools[dev], &props);
      if (e != cudaSuccess) {
        g_pools[dev] = nullptr;
        return e;
      }
      unsigned long long keep = ~0ull;
      cudaMemPoolSetAttribute(g_pools[dev], cudaMemPoolAttrReleaseThreshold, &keep);
    }
    pool = g_pools[dev];
  }
  e = cudaMallocFromPoolAsync(p, bytes, pool, s);
  if (e == cudaErrorMemoryAllocation) {
    // Freed blocks the pool keeps may be what is missing: once the stream has
    // passed its pending frees, give them back to the device and try once more.
    cudaGetLastError();
    if (cudaStreamSynchronize(s) == cudaSuccess) {
      cudaMemPoolTrimTo(pool, 0);
      e = cudaMallocFromPoolAsync(p, bytes, pool, s);
    }
  }
  // a failed allocation leaves no error behind for the next CUDA call of the
  // process (another library would otherwise report it as its own)
  if (e != cudaSuccess) cudaGetLastError();
  return e;
}

void pool_trim_all() {
  std::lock_guard<std::mutex> g(g_pool_mu);
  for (int d = 0; d < 64; d++)
    if (g_pools[d]) cudaMemPoolTrimTo(g_pools[d], 0);
}
}  // namespace dg

extern "C" int dg_release_memory(void) {
  dg::device_state().release_idle_workspaces();
  dg::pool_trim_all();
  return 0;
}

extern "C" int dg_finalize(void) {
  dg::clear_graphs();
  dg::device_state().release_idle_workspaces();
  dg::pool_trim_all();
  return 0;
}

extern "C" long long dg_kernel_launches(void) { return dg::launches(); }

extern "C" int dg_set_device(int device) {
  DG_CUDA_TRY(cudaSetDevice(device));
  return 0;
}

extern "C" int dg_device_alloc(size_t bytes, void **out) {
  DG_CHECK_ARG(out != nullptr, 2);
  *out = nullptr;
  if (bytes == 0) return 0;
  if (cudaMalloc(out, bytes) != cudaSuccess) {
    cudaGetLastError();
    dg_set_last_error(__FILE__, __LINE__, "cudaMalloc failed");
    return DG_ERR_NOMEM;
  }
  return 0;
}

extern "C" int dg_device_free(void *p) {
  if (p) DG_CUDA_TRY(cudaFree(p));
  return 0;
}

extern "C" int dg_host_alloc(size_t bytes, void **out) {
  DG_CHECK_ARG(out != nullptr, 2);
  *out = nullptr;
  if (bytes == 0) return 0;
  if (cudaHostAlloc(out, bytes, cudaHostAllocMapped | cudaHostAllocPortable) != cudaSuccess) {
    cudaGetLastError();
    dg_set_last_error(__FILE__, __LINE__, "cudaHostAlloc failed");
    return DG_ERR_NOMEM;
  }
  return 0;
}

extern "C" int dg_host_free(void *p) {
  if (p) DG_CUDA_TRY(cudaFreeHost(p));
  return 0;
}

extern "C" int dg_copy(void *dst, const void *src, size_t bytes, int kind, void *stream) {
  DG_CHECK_ARG(kind >= 0 && kind <= 2, 4);
  static const cudaMemcpyKind kinds[3] = {cudaMemcpyHostToDevice, cudaMemcpyDeviceToHost,
                                          cudaMemcpyDeviceToDevice};
  if (bytes == 0) return 0;
  DG_CUDA_TRY(cudaMemcpyAsync(dst, src, bytes, kinds[kind], (cudaStream_t)stream));
  return 0;
}

extern "C" int dg_stream_create(void **out) {
  DG_CHECK_ARG(out != nullptr, 1);
  cudaStream_t s;
  DG_CUDA_TRY(cudaStreamCreateWithFlags(&s, cudaStreamNonBlocking));
  *out = (void *)s;
  return 0;
}

extern "C" int dg_stream_destroy(void *stream) {
  if (stream) DG_CUDA_TRY(cudaStreamDestroy((cudaStream_t)stream));
  return 0;
}

extern "C" int dg_stream_synchronize(void *stream) {
  DG_CUDA_TRY(cudaStreamSynchronize((cudaStream_t)stream));
  return 0;
}

extern "C" int dg_set_f64_engine(int engine) {
  int old = dg::get_f64_engine();
  dg::set_f64_engine(engine);
  return old;
}

extern "C" int dg_get_f64_engine(void) { return dg::get_f64_engine(); }

extern "C" int dg_potrf_async(char uplo, int n, double *A, int lda, int *info_dev, void *stream) {
  DG_CHECK_ARG(is_one_of(uplo, "ULul"), 1);
  DG_CHECK_ARG(n >= 0, 2);
  DG_CHECK_ARG(lda >= (n > 1 ? n : 1), 4);
  DG_CHECK_ARG(info_dev != nullptr, 5);
  return dg::potrf_f64(uplo, n, A, lda, info_dev, 0, (cudaStream_t)stream);
}

extern "C" int dg_potrf(char uplo, int n, double *A, int lda, int *info_host, void *stream) {
  DG_CHECK_ARG(is_one_of(uplo, "ULul"), 1);
  DG_CHECK_ARG(n >= 0, 2);
  DG_CHECK_ARG(lda >= (n > 1 ? n : 1), 4);
  cudaStream_t s = (cudaStream_t)stream;
  int *info = nullptr;
  int rc = dg::device_state().scratch_int(&info);
  if (rc) return rc;
  DG_CUDA_TRY(cudaMemsetAsync(info, 0, sizeof(int), s));
  rc = dg::potrf_f64(uplo, n, A, lda, info, 0, s);
  if (rc) return rc;
  if (!info_host) return 0;
  int h = dg::read_info(info, s);
  *info_host = h;
  return h;
}

extern "C" int dg_trsm(char side, char uplo, char transa, char diag, int m, int n, double alpha,
                       const double *A, int lda, double *B, int ldb, void *stream) {
  DG_CHECK_ARG(is_one_of(side, "LRlr"), 1);
  DG_CHECK_ARG(is_one_of(uplo, "ULul"), 2);
  DG_CHECK_ARG(is_one_of(transa, "NTCntc"), 3);
  DG_CHECK_ARG(is_one_of(diag, "NUnu"), 4);
  DG_CHECK_ARG(m >= 0, 5);
  DG_CHECK_ARG(n >= 0, 6);
  int ka = (side == 'L' || side == 'l') ? m : n;
  DG_CHECK_ARG(lda >= (ka > 1 ? ka : 1), 9);
  DG_CHECK_ARG(ldb >= (m > 1 ? m : 1), 11);
  return dg::trsm_f64(side, uplo, transa, diag, m, n, alpha, A, lda, B, ldb, nullptr,
                      (cudaStream_t)stream);
}

extern "C" int dg_syrk(char uplo, char trans, int n, int k, double alpha, const double *A, int lda,
                       double beta, double *C, int ldc, void *stream) {
  DG_CHECK_ARG(is_one_of(uplo, "ULul"), 1);
  DG_CHECK_ARG(is_one_of(trans, "NTCntc"), 2);
  DG_CHECK_ARG(n >= 0, 3);
  DG_CHECK_ARG(k >= 0, 4);
  bool nt = (trans == 'N' || trans == 'n');
  int ra = nt ? n : k;
  DG_CHECK_ARG(lda >= (ra > 1 ? ra : 1), 7);
  DG_CHECK_ARG(ldc >= (n > 1 ? n : 1), 10);
  dg::Tri tri = (uplo == 'U' || uplo == 'u') ? dg::TRI_UPPER : dg::TRI_LOWER;
  return dg::gemm_f64(nt ? 'N' : 'T', nt ? 'T' : 'N', n, n, k, alpha, A, lda, A, lda, beta, C, ldc,
                      tri, nullptr, (cudaStream_t)stream);
}

extern "C" int dg_gemm(char transa, char transb, int m, int n, int k, double alpha,
                       const double *A, int lda, const double *B, int ldb, double beta, double *C,
                       int ldc, void *stream) {
  DG_CHECK_ARG(is_one_of(transa, "NTCntc"), 1);
  DG_CHECK_ARG(is_one_of(transb, "NTCntc"), 2);
  DG_CHECK_ARG(m >= 0, 3);
  DG_CHECK_ARG(n >= 0, 4);
  DG_CHECK_ARG(k >= 0, 5);
  bool na = (transa == 'N' || transa == 'n'), nb = (transb == 'N' || transb == 'n');
  int ra = na ? m : k, rb = nb ? k : n;
  DG_CHECK_ARG(lda >= (ra > 1 ? ra : 1), 8);
  DG_CHECK_ARG(ldb >= (rb > 1 ? rb : 1), 10);
  DG_CHECK_ARG(ldc >= (m > 1 ? m : 1), 13);
  return dg::gemm_f64(transa, transb, m, n, k, alpha, A, lda, B, ldb, beta, C, ldc, dg::TRI_NONE,
                      nullptr, (cudaStream_t)stream);
}

extern "C" int dg_trsv(char uplo, char trans, char diag, int n, const double *A, int lda, double *x,
                       void *stream) {
  DG_CHECK_ARG(is_one_of(uplo, "ULul"), 1);
  DG_CHECK_ARG(is_one_of(trans, "NTCntc"), 2);
  DG_CHECK_ARG(is_one_of(diag, "NUnu"), 3);
  DG_CHECK_ARG(n >= 0, 4);
  DG_CHECK_ARG(lda >= (n > 1 ? n : 1), 6);
  return dg::trsm_f64('L', uplo, trans, diag, n, 1, 1.0, A, lda, x, n > 1 ? n : 1, nullptr,
                      (cudaStream_t)stream);
}

extern "C" int dg_gemv(char trans, int m, int n, double alpha, const double *A, int lda,
                       const double *x, double beta, double *y, void *stream) {
  DG_CHECK_ARG(is_one_of(trans, "NTCntc"), 1);
  DG_CHECK_ARG(m >= 0, 2);
  DG_CHECK_ARG(n >= 0, 3);
  DG_CHECK_ARG(lda >= (m > 1 ? m : 1), 6);
  bool nt = (trans == 'N' || trans == 'n');
  int rows = nt ? m : n, inner = nt ? n : m;
  return dg::gemm_f64(nt ? 'N' : 'T', 'N', rows, 1, inner, alpha, A, lda, x, inner > 1 ? inner : 1,
                      beta, y, rows > 1 ? rows : 1, dg::TRI_NONE, nullptr, (cudaStream_t)stream);
}

// ---------------------------------------------------------------------------
// whole-call entry points
// ---------------------------------------------------------------------------
namespace dg {

// The factorization's slots, plus three columns of slots so that a following
// solve with up to nb right-hand sides finds its ring in place (with the
// inverses: oz_solve_ring_bytes_for(n, nb, nb, true)), then the FP64
// inverses of the last kOzRingDepth diagonal tiles.
static size_t oz_inv_offset(int n, int nb) {
  const int mt = (n + nb - 1) / nb;
  return (size_t)kOzRingDepth * (mt + 3) * oz_slot_bytes((nb + 7) / 8 * 8, nb);
}
static size_t oz_inv_bytes(int nb) { return ((size_t)nb * nb * 8 + 255) & ~(size_t)255; }
size_t oz_ring_bytes_for(int n, int nb) {
  return oz_inv_offset(n, nb) + (size_t)kOzRingDepth * oz_inv_bytes(nb);
}

// The emulated-FP64 form of the same task graph: after TRSM(k, j) a split
// task cuts tile (k, j)'s vectors into BF16 slices once, into ring slot
// (k mod depth, j), and every SYRK/GEMM of step k reads its operands from the
// slots.  The datadeps rules order a slot's reuse after its last reader.
static void build_cholesky_region_oz(dg_region *r, bool up, int n, int nb, double *const *tiles,
                                     void *ring, double *winv) {
  const int mt = (n + nb - 1) / nb;
  auto rows = [&](int i) { return (i + 1) * nb <= n ? nb : n - i * nb; };
  auto T = [&](int i, int j) { return tiles[i + (size_t)j * mt]; };
  const int ldk = (nb + 7) / 8 * 8;
  const size_t sb = oz_slot_bytes(ldk, nb);
  auto slot = [&](int k, int j) {
    return (double *)((char *)ring + ((size_t)(k % kOzRingDepth) * mt + j) * sb);
  };
  // The panel solve of step k (cholesky.jl:40-42 / 85-87) runs as emulated
  // GEMMs with the inverse of the diagonal factor: W = U_kk^-T (upper) or
  // L_kk^-T (lower) is formed once by substitution on the identity, and each
  // panel tile becomes W A(k, j) (upper) or A(j, k) W (lower).  POTRF(k) and
  // the inversion cut their recursions' operands into slices in slot (k, k),
  // which then holds W's slices; slot (k, j) holds the panel tile's input
  // slices, then its result's for the trailing update.
  const int slot_units = (int)(sb / 256);
  auto W = [&](int k) {
    if (winv) return winv + (size_t)k * nb * nb;
    return (double *)((char *)ring + oz_inv_offset(n, nb) + (size_t)(k % kOzRingDepth) * oz_inv_bytes(nb));
  };
  // W_k of an n x n tile with n >= 256 by halves (h + n2 = n): the two
  // diagonal inverses by substitution, side by side, and the off-diagonal
  // block as two emulated products,
  //   upper: W = [W11 0; -W22 (U12' W11)  W22],
  //   lower: W = [W11 -W11 (L21' W22); 0  W22],
  // the product's operands cut into three sub-slots of slot (k, k) (the slot
  // then receives W's own slices).  A quarter of the substitution's FP64 work.
  auto add_inv = [&](int k) {
    const int nk = rows(k);
    double *Wk = W(k);
    const double *Uk = T(k, k);
    dg_task t;
    const int h0 = ((nk / 2) + 63) / 64 * 64, cap0 = h0 > nk - h0 ? h0 : nk - h0;
    if (nk < 256 || 3 * oz_slot_bytes((cap0 + 7) / 8 * 8, cap0) > sb) {
      memset(&t, 0, sizeof t);
      t.op = OP_OZ_INV; t.uplo = up ? 'U' : 'L'; t.n = nk; t.a = Uk; t.lda = nk;
      t.c = Wk; t.ldc = nk; t.b = slot(k, k); t.ldb = slot_units;
      dg_region_add(r, &t);
      mark_urgent(r);
      return;
    }
    const int h = h0, n2 = nk - h;
    const int cap = cap0, ldh = (cap + 7) / 8 * 8;
    const size_t subb = oz_slot_bytes(ldh, cap);
    auto sub = [&](int i) { return (double *)((char *)slot(k, k) + (size_t)i * subb); };
    auto add = [&]() { dg_region_add(r, &t); mark_urgent(r); };
    // the zero block: upper W12 (rows 0..h-1, columns h..), lower W21
    memset(&t, 0, sizeof t);
    t.op = OP_OZ_ZERO; t.c = up ? Wk + (size_t)h * nk : Wk + h; t.ldc = nk;
    t.m = up ? h : n2; t.n = up ? n2 : h;
    add();
    for (int half = 0; half < 2; half++) {  // W11, W22
      const size_t off = half ? (size_t)h + (size_t)h * nk : 0;
      memset(&t, 0, sizeof t);
      t.op = OP_OZ_INV; t.uplo = up ? 'U' : 'L'; t.n = half ? n2 : h; t.a = Uk + off; t.lda = nk;
      t.c = Wk + off; t.ldc = nk;
      add();
    }
    auto split = [&](const double *src, int K, int nv, char trans, double *dst) {
      memset(&t, 0, sizeof t);
      t.op = OP_OZ_SPLIT; t.a = src; t.lda = nk; t.m = K; t.n = nv; t.trans = trans;
      t.c = dst; t.ldc = ldh; t.k = cap;
      add();
    };
    auto gemm = [&](int m, int nn, int K, double alpha, double *a, double *b, double *c) {
      memset(&t, 0, sizeof t);
      t.op = OP_OZ_GEMM; t.uplo = 'N'; t.m = m; t.n = nn; t.k = K; t.alpha = alpha; t.beta = 0.0;
      t.a = a; t.b = b; t.lda = ldh; t.ldb = cap; t.c = c; t.ldc = nk;
      add();
    };
    const double *W11 = Wk, *W22 = Wk + (size_t)h + (size_t)h * nk;
    if (up) {
      double *W21 = Wk + h;  // T = U12' W11 there first
      split(Uk + (size_t)h * nk, h, n2, 'N', sub(0));  // columns of U12
      split(W11, h, h, 'N', sub(1));                    // columns of W11
      gemm(n2, h, h, 1.0, sub(0), sub(1), W21);
      split(W22, n2, n2, 'T', sub(2));                  // rows of W22
      split(W21, n2, h, 'N', sub(0));                   // columns of T
      gemm(n2, h, n2, -1.0, sub(2), sub(0), W21);
    } else {
      double *W12 = Wk + (size_t)h * nk;  // T = L21' W22 there first
      split(Uk + h, n2, h, 'N', sub(0));                // columns of L21
      split(W22, n2, n2, 'N', sub(1));                  // columns of W22
      gemm(h, n2, n2, 1.0, sub(0), sub(1), W12);
      split(W11, h, h, 'T', sub(2));                    // rows of W11
      split(W12, h, n2, 'N', sub(0));                   // columns of T
      gemm(h, n2, h, -1.0, sub(2), sub(0), W12);
    }
  };
  for (int k = 0; k < mt; k++) {
    dg_task t;
    memset(&t, 0, sizeof t);
    t.op = OP_OZ_POTRF; t.uplo = up ? 'U' : 'L'; t.n = rows(k); t.c = T(k, k); t.ldc = rows(k);
    t.info_offset = k * nb; t.b = slot(k, k); t.ldb = slot_units;
    dg_region_add(r, &t);
    mark_urgent(r);
    if (k + 1 == mt) {
      if (winv) add_inv(k);  // kept for the solves: the last tile's inverse too
      break;
    }
    add_inv(k);
    // rows of W (upper: A-vectors) / columns (lower: B-vectors); W's diagonal
    // 1/u_ii dominates its vectors, so it stays FP64 and scales the panel
    // tile exactly, and only the off-diagonal part is sliced
    memset(&t, 0, sizeof t);
    t.op = OP_OZ_SPLIT; t.a = W(k); t.lda = rows(k); t.m = rows(k); t.n = rows(k);
    t.trans = up ? 'T' : 'N'; t.diag = 'Z'; t.c = slot(k, k); t.ldc = ldk; t.k = nb;
    dg_region_add(r, &t);
    mark_urgent(r);
    // Priority of a tile of column j (row j for 'L') at step k: j - k - 1,
    // the number of steps before POTRF(j) needs it, so the work needed soonest
    // runs first; a task's level is never above those of its inputs.
    for (int j = k + 1; j < mt; j++) {
      const int lvl = j - k - 1;
      for (int pass = 0; pass < 2; pass++) {  // the tile's input, then its result
        memset(&t, 0, sizeof t);
        t.op = OP_OZ_SPLIT; t.m = rows(k); t.n = rows(j); t.c = slot(k, j); t.ldc = ldk; t.k = nb;
        if (up) {  // columns of A(k, j) / U(k, j)
          t.trans = 'N'; t.a = T(k, j); t.lda = rows(k);
        } else {   // rows of A(j, k) / L(j, k)
          t.trans = 'T'; t.a = T(j, k); t.lda = rows(j);
        }
        dg_region_add(r, &t);
        mark_level(r, lvl);
        if (pass == 1) break;
        memset(&t, 0, sizeof t);
        t.op = OP_OZ_GEMM; t.uplo = 'N'; t.k = rows(k); t.alpha = 1.0; t.beta = 0.0;
        t.lda = ldk; t.ldb = nb;
        if (up) {  // U(k, j) = diag(W) A(k, j) + offdiag(W) A(k, j)
          t.m = rows(k); t.n = rows(j); t.a = slot(k, k); t.b = slot(k, j);
          t.c = T(k, j); t.ldc = rows(k); t.side = 'A';
        } else {   // L(j, k) = A(j, k) diag(W) + A(j, k) offdiag(W)
          t.m = rows(j); t.n = rows(k); t.a = slot(k, j); t.b = slot(k, k);
          t.c = T(j, k); t.ldc = rows(j); t.side = 'B';
        }
        if (lvl > 0) t.diag = 'P';  // off the critical path: one CTA per several blocks
        dg_region_add(r, &t);
        mark_level(r, lvl);
      }
    }
    // cholesky.jl:43-52 (upper) / 88-97 (lower): C(m, j) -= V_m' V_j over the
    // vectors V of step k; the diagonal tiles keep one triangle (SYRK).
    for (int m = k + 1; m < mt; m++) {
      for (int j = m; j < mt; j++) {
        memset(&t, 0, sizeof t);
        t.op = OP_OZ_GEMM; t.k = rows(k); t.alpha = -1.0; t.beta = 1.0;
        t.lda = ldk; t.ldb = nb;
        if (up) {
          t.m = rows(m); t.n = rows(j); t.a = slot(k, m); t.b = slot(k, j);
          t.c = T(m, j); t.ldc = rows(m); t.uplo = (j == m) ? 'U' : 'N';
        } else {
          t.m = rows(j); t.n = rows(m); t.a = slot(k, j); t.b = slot(k, m);
          t.c = T(j, m); t.ldc = rows(j); t.uplo = (j == m) ? 'L' : 'N';
        }
        // level j - k - 1 as for the panel tiles; off the critical path the
        // tiles share the GPU, one CTA per several output blocks
        const int lvl = j - k - 1;
        if (lvl > 0) t.diag = 'P';
        dg_region_add(r, &t);
        mark_level(r, lvl);
      }
    }
  }
}

void build_upload_tasks(dg_region *r, char uplo, int n, int nb, double *const *tiles,
                        const double *host, long long ldh) {
  const int mt = (n + nb - 1) / nb;
  const bool up = (uplo == 'U' || uplo == 'u');
  auto rows = [&](int i) { return (i + 1) * nb <= n ? nb : n - i * nb; };
  // on the transfer streams in the order of first use: the factor's
  // triangle by column (row for 'L'), then the other triangle
  for (int pass = 0; pass < 2; pass++)
    for (int j = 0; j < mt; j++)
      for (int i = 0; i < mt; i++) {
        const int a = up ? i : j, b = up ? j : i;  // row and column of the upper form
        const bool mine = a <= b;
        if (mine != (pass == 0)) continue;
        dg_task t;
        memset(&t, 0, sizeof t);
        t.op = OP_UPLOAD; t.m = rows(i); t.n = rows(j);
        t.a = host + (size_t)i * nb * ldh + (size_t)j * nb; t.lda = (int)ldh;
        t.c = tiles[i + (size_t)j * mt]; t.ldc = rows(i);
        dg_region_add(r, &t);
        mark_transfer(r);
      }
}

// ---------------------------------------------------------------------------
// gemm_dagger! / syrk_dagger! + copytri! (src/array/mul.jl:133-425)
// ---------------------------------------------------------------------------
size_t mul_ring_bytes_for(int m, int n, int nb) {
  const int mt = (m + nb - 1) / nb, nt = (n + nb - 1) / nb;
  return (size_t)kOzRingDepth * (mt + nt) * oz_slot_bytes((nb + 7) / 8 * 8, nb);
}

namespace {
struct MulGrid {
  int nb;
  int len(int i, int total) const { return (i + 1) * nb <= total ? nb : total - i * nb; }
};
}  // namespace

// The rows of op(X) block (i, p) of a tile grid holding X (op = 'N': X is
// rows x K with tile (i, p); 'T': X is K x rows with tile (p, i)) cut into
// slot `dst` as vectors of length K.
static void add_row_split(dg_region *r, const MulGrid &g, bool tr, double *const *X, int rows,
                          int K, int i, int p, double *dst, int ldk) {
  const int mt = (rows + g.nb - 1) / g.nb, kt = (K + g.nb - 1) / g.nb;
  dg_task t;
  memset(&t, 0, sizeof t);
  t.op = OP_OZ_SPLIT; t.m = g.len(p, K); t.n = g.len(i, rows);
  if (!tr) {  // rows of X(i, p)
    t.a = X[i + (size_t)p * mt]; t.lda = g.len(i, rows); t.trans = 'T';
  } else {    // columns of X(p, i)
    t.a = X[p + (size_t)i * kt]; t.lda = g.len(p, K); t.trans = 'N';
  }
  t.c = dst; t.ldc = ldk; t.k = g.nb;
  dg_region_add(r, &t);
}

// The transposes of copytri!: tile (j, i) = tile (i, j)' for i < j, the
// diagonal tiles' upper triangles mirrored.
static void add_copytri(dg_region *r, const MulGrid &g, int n, double *const *C) {
  const int nt = (n + g.nb - 1) / g.nb;
  for (int i = 0; i < nt; i++)
    for (int j = i; j < nt; j++) {
      dg_task t;
      memset(&t, 0, sizeof t);
      if (i == j) {
        t.op = OP_TILE_MIRROR; t.n = g.len(i, n); t.c = C[i + (size_t)i * nt]; t.ldc = g.len(i, n);
      } else {
        t.op = OP_TILE_T; t.m = g.len(i, n); t.n = g.len(j, n);
        t.a = C[i + (size_t)j * nt]; t.lda = g.len(i, n);
        t.c = C[j + (size_t)i * nt]; t.ldc = g.len(j, n);
      }
      dg_region_add(r, &t);
    }
}

void build_gemm_region(dg_region *r, char ta, char tb, int m, int n, int k, int nb, double alpha,
                       double *const *A, double *const *B, double beta, double *const *C,
                       void *oz_ring) {
  const MulGrid g{nb};
  const int mt = (m + nb - 1) / nb, nt = (n + nb - 1) / nb, kt = (k + nb - 1) / nb;
  const bool tA = !(ta == 'N' || ta == 'n'), tB = !(tb == 'N' || tb == 'n');
  auto Ct = [&](int i, int j) { return C[i + (size_t)j * mt]; };
  if (!oz_ring) {
    // mul.jl:154-212: for each C tile, the k loop of gemm! with beta on the first
    for (int i = 0; i < mt; i++)
      for (int j = 0; j < nt; j++)
        for (int p = 0; p < kt; p++) {
          dg_task t;
          memset(&t, 0, sizeof t);
          t.op = DG_OP_GEMM; t.transa = tA ? 'T' : 'N'; t.transb = tB ? 'T' : 'N';
          t.m = g.len(i, m); t.n = g.len(j, n); t.k = g.len(p, k);
          t.alpha = alpha; t.beta = (p == 0) ? beta : 1.0;
          t.a = tA ? A[p + (size_t)i * kt] : A[i + (size_t)p * mt];
          t.lda = tA ? g.len(p, k) : g.len(i, m);
          t.b = tB ? B[j + (size_t)p * nt] : B[p + (size_t)j * kt];
          t.ldb = tB ? g.len(j, n) : g.len(p, k);
          t.c = Ct(i, j); t.ldc = g.len(i, m);
          dg_region_add(r, &t);
        }
    return;
  }
  // emulated: step p cuts op(A)'s block column p and op(B)'s block row p into
  // slices once, then every C tile takes its product (the same order of the
  // k accumulation per tile)
  const int ldk = (nb + 7) / 8 * 8;
  const size_t sb = oz_slot_bytes(ldk, nb);
  auto slot = [&](int p, int q) {
    return (double *)((char *)oz_ring + ((size_t)(p % kOzRingDepth) * (mt + nt) + q) * sb);
  };
  for (int p = 0; p < kt; p++) {
    for (int i = 0; i < mt; i++) add_row_split(r, g, tA, A, m, k, i, p, slot(p, i), ldk);
    // the columns of op(B) block (p, j) are the rows of op(B)' block (j, p)
    for (int j = 0; j < nt; j++) add_row_split(r, g, !tB, B, n, k, j, p, slot(p, mt + j), ldk);
    for (int i = 0; i < mt; i++)
      for (int j = 0; j < nt; j++) {
        dg_task t;
        memset(&t, 0, sizeof t);
        t.op = OP_OZ_GEMM; t.uplo = 'N'; t.diag = 'P';
        t.m = g.len(i, m); t.n = g.len(j, n); t.k = g.len(p, k);
        t.alpha = alpha; t.beta = (p == 0) ? beta : 1.0;
        t.a = slot(p, i); t.b = slot(p, mt + j); t.lda = ldk; t.ldb = nb;
        t.c = Ct(i, j); t.ldc = g.len(i, m);
        dg_region_add(r, &t);
      }
  }
}

void build_syrk_region(dg_region *r, char trans, int n, int k, int nb, double alpha,
                       double *const *A, double beta, double *const *C, void *oz_ring) {
  const MulGrid g{nb};
  const int nt = (n + nb - 1) / nb, kt = (k + nb - 1) / nb;
  const bool tr = !(trans == 'N' || trans == 'n');
  auto Ct = [&](int i, int j) { return C[i + (size_t)j * nt]; };
  // op(A) block (i, p): A(i, p) ('N', A is n x k) or A(p, i)' ('T', A is k x n)
  auto At = [&](int i, int p) { return tr ? A[p + (size_t)i * kt] : A[i + (size_t)p * nt]; };
  auto Ald = [&](int i, int p) { return tr ? g.len(p, k) : g.len(i, n); };
  if (!oz_ring) {
    // mul.jl:244-361 with uplo = 'U': syrk! on the diagonal tiles, gemm! on
    // the upper ones, beta on the first term of each
    for (int j = 0; j < nt; j++) {
      for (int p = 0; p < kt; p++) {
        dg_task t;
        memset(&t, 0, sizeof t);
        t.op = DG_OP_SYRK; t.uplo = 'U'; t.trans = tr ? 'T' : 'N';
        t.n = g.len(j, n); t.k = g.len(p, k); t.alpha = alpha; t.beta = (p == 0) ? beta : 1.0;
        t.a = At(j, p); t.lda = Ald(j, p); t.c = Ct(j, j); t.ldc = g.len(j, n);
        dg_region_add(r, &t);
      }
      for (int m2 = j + 1; m2 < nt; m2++)
        for (int p = 0; p < kt; p++) {
          dg_task t;
          memset(&t, 0, sizeof t);
          t.op = DG_OP_GEMM; t.transa = tr ? 'T' : 'N'; t.transb = tr ? 'N' : 'T';
          t.m = g.len(j, n); t.n = g.len(m2, n); t.k = g.len(p, k);
          t.alpha = alpha; t.beta = (p == 0) ? beta : 1.0;
          t.a = At(j, p); t.lda = Ald(j, p); t.b = At(m2, p); t.ldb = Ald(m2, p);
          t.c = Ct(j, m2); t.ldc = g.len(j, n);
          dg_region_add(r, &t);
        }
    }
  } else {
    const int ldk = (nb + 7) / 8 * 8;
    const size_t sb = oz_slot_bytes(ldk, nb);
    auto slot = [&](int p, int q) {
      return (double *)((char *)oz_ring + ((size_t)(p % kOzRingDepth) * (nt + 0) + q) * sb);
    };
    for (int p = 0; p < kt; p++) {
      for (int i = 0; i < nt; i++) add_row_split(r, g, tr, A, n, k, i, p, slot(p, i), ldk);
      for (int i = 0; i < nt; i++)
        for (int j = i; j < nt; j++) {
          dg_task t;
          memset(&t, 0, sizeof t);
          t.op = OP_OZ_GEMM; t.uplo = (i == j) ? 'U' : 'N'; t.diag = 'P';
          t.m = g.len(i, n); t.n = g.len(j, n); t.k = g.len(p, k);
          t.alpha = alpha; t.beta = (p == 0) ? beta : 1.0;
          t.a = slot(p, i); t.b = slot(p, j); t.lda = ldk; t.ldb = nb;
          t.c = Ct(i, j); t.ldc = g.len(i, n);
          dg_region_add(r, &t);
        }
    }
  }
  add_copytri(r, g, n, C);  // mul.jl:363
}

void build_cholesky_region(dg_region *r, char uplo, int n, int nb, double *const *tiles,
                           void *oz_ring, double *winv) {
  const int mt = (n + nb - 1) / nb;
  auto rows = [&](int i) { return (i + 1) * nb <= n ? nb : n - i * nb; };
  auto T = [&](int i, int j) { return tiles[i + (size_t)j * mt]; };
  const bool up = (uplo == 'U' || uplo == 'u');
  if (oz_ring) {
    build_cholesky_region_oz(r, up, n, nb, tiles, oz_ring, winv);
    return;
  }
  for (int k = 0; k < mt; k++) {
    dg_task t;
    memset(&t, 0, sizeof t);
    t.op = DG_OP_POTRF; t.uplo = up ? 'U' : 'L'; t.n = rows(k); t.c = T(k, k); t.ldc = rows(k);
    t.info_offset = k * nb;
    dg_region_add(r, &t);
    if (up) {
      for (int j = k + 1; j < mt; j++) {  // cholesky.jl:40-42
        memset(&t, 0, sizeof t);
        t.op = DG_OP_TRSM; t.side = 'L'; t.uplo = 'U'; t.transa = 'T'; t.diag = 'N';
        t.m = rows(k); t.n = rows(j); t.alpha = 1.0;
        t.a = T(k, k); t.lda = rows(k); t.c = T(k, j); t.ldc = rows(k);
        dg_region_add(r, &t);
      }
      for (int m = k + 1; m < mt; m++) {  // cholesky.jl:43-52
        memset(&t, 0, sizeof t);
        t.op = DG_OP_SYRK; t.uplo = 'U'; t.trans = 'T'; t.n = rows(m); t.k = rows(k);
        t.alpha = -1.0; t.beta = 1.0; t.a = T(k, m); t.lda = rows(k); t.c = T(m, m); t.ldc = rows(m);
        dg_region_add(r, &t);
        for (int j = m + 1; j < mt; j++) {
          memset(&t, 0, sizeof t);
          t.op = DG_OP_GEMM; t.transa = 'T'; t.transb = 'N'; t.m = rows(m); t.n = rows(j);
          t.k = rows(k); t.alpha = -1.0; t.beta = 1.0; t.a = T(k, m); t.lda = rows(k);
          t.b = T(k, j); t.ldb = rows(k); t.c = T(m, j); t.ldc = rows(m);
          dg_region_add(r, &t);
        }
      }
    } else {
      for (int m = k + 1; m < mt; m++) {  // cholesky.jl:85-87
        memset(&t, 0, sizeof t);
        t.op = DG_OP_TRSM; t.side = 'R'; t.uplo = 'L'; t.transa = 'T'; t.diag = 'N';
        t.m = rows(m); t.n = rows(k); t.alpha = 1.0;
        t.a = T(k, k); t.lda = rows(k); t.c = T(m, k); t.ldc = rows(m);
        dg_region_add(r, &t);
      }
      for (int j = k + 1; j < mt; j++) {  // cholesky.jl:88-97
        memset(&t, 0, sizeof t);
        t.op = DG_OP_SYRK; t.uplo = 'L'; t.trans = 'N'; t.n = rows(j); t.k = rows(k);
        t.alpha = -1.0; t.beta = 1.0; t.a = T(j, k); t.lda = rows(j); t.c = T(j, j); t.ldc = rows(j);
        dg_region_add(r, &t);
        for (int m = j + 1; m < mt; m++) {
          memset(&t, 0, sizeof t);
          t.op = DG_OP_GEMM; t.transa = 'N'; t.transb = 'T'; t.m = rows(m); t.n = rows(j);
          t.k = rows(k); t.alpha = -1.0; t.beta = 1.0; t.a = T(m, k); t.lda = rows(m);
          t.b = T(j, k); t.ldb = rows(j); t.c = T(m, j); t.ldc = rows(m);
          dg_region_add(r, &t);
        }
      }
    }
  }
}

// One left-side block solve of trsm.jl:89-140 (alpha = 1) over the factor's
// tiles and the right-hand side's tiles.
size_t oz_solve_ring_bytes_for(int n, int nb, int nrhs, bool inv) {
  const int mt = (n + nb - 1) / nb, bnt = (nrhs + nb - 1) / nb;
  return (size_t)kOzRingDepth * (mt + bnt + (inv ? 1 + bnt : 0)) *
         oz_slot_bytes((nb + 7) / 8 * 8, nb);
}

void build_solve_pass(dg_region *r, char uplo, char trans, int n, int nb, double *const *tiles,
                      int nrhs, double *const *btiles, void *oz_ring, int step0,
                      const double *winv, char diag) {
  const int mt = (n + nb - 1) / nb, bnt = (nrhs + nb - 1) / nb;
  auto rows = [&](int i) { return (i + 1) * nb <= n ? nb : n - i * nb; };
  auto cols = [&](int j) { return (j + 1) * nb <= nrhs ? nb : nrhs - j * nb; };
  auto A = [&](int i, int j) { return tiles[i + (size_t)j * mt]; };
  auto B = [&](int i, int j) { return btiles[i + (size_t)j * mt]; };
  const bool forward = (uplo == 'U') ? (trans != 'N') : (trans == 'N');
  // emulated form: slots (step mod depth, m) hold the A-vectors of one
  // update, slots depth*mt + (step mod depth)*bnt + c the solved block's
  // columns; the datadeps rules order each slot's reuse after its readers
  const int ldk = (nb + 7) / 8 * 8;
  const size_t sb = oz_slot_bytes(ldk, nb);
  auto aslot = [&](int step, int m) {
    return (double *)((char *)oz_ring + ((size_t)(step % kOzRingDepth) * mt + m) * sb);
  };
  auto xslot = [&](int step, int c) {
    return (double *)((char *)oz_ring +
                      ((size_t)kOzRingDepth * mt + (size_t)(step % kOzRingDepth) * bnt + c) * sb);
  };
  // with the inverses: slots after those hold the inverse's vectors and the
  // block's columns before its solve
  const size_t inv0 = (size_t)kOzRingDepth * (mt + bnt);
  auto wslot = [&](int step) {
    return (double *)((char *)oz_ring + (inv0 + (size_t)(step % kOzRingDepth)) * sb);
  };
  auto bslot = [&](int step, int c) {
    return (double *)((char *)oz_ring +
                      (inv0 + kOzRingDepth + (size_t)(step % kOzRingDepth) * bnt + c) * sb);
  };
  const bool inv = (oz_ring != nullptr && winv != nullptr);
  for (int s = 0; s < mt; s++) {
    int k = forward ? s : mt - 1 - s;
    if (inv) {
      // op(A(k, k))^-1 is W_k (trans 'T') or W_k' ('N'), W_k = U_kk^-T or
      // L_kk^-T: its rows are W_k's rows or columns, its diagonal stays FP64
      dg_task t;
      memset(&t, 0, sizeof t);
      t.op = OP_OZ_SPLIT; t.a = winv + (size_t)k * nb * nb; t.lda = rows(k); t.m = rows(k);
      t.n = rows(k); t.trans = (trans == 'N') ? 'N' : 'T'; t.diag = 'Z';
      t.c = wslot(step0 + s); t.ldc = ldk; t.k = nb;
      dg_region_add(r, &t);
    }
    for (int c = 0; c < bnt; c++) {
      dg_task t;
      memset(&t, 0, sizeof t);
      if (inv) {
        // B(k, c) = op(A(k, k))^-1 B(k, c) as one emulated product
        t.op = OP_OZ_SPLIT; t.trans = 'N'; t.a = B(k, c); t.lda = rows(k); t.m = rows(k);
        t.n = cols(c); t.c = bslot(step0 + s, c); t.ldc = ldk; t.k = nb;
        dg_region_add(r, &t);
        mark_urgent(r);
        memset(&t, 0, sizeof t);
        t.op = OP_OZ_GEMM; t.uplo = 'N'; t.m = rows(k); t.n = cols(c); t.k = rows(k);
        t.alpha = 1.0; t.beta = 0.0; t.a = wslot(step0 + s); t.b = bslot(step0 + s, c);
        t.lda = ldk; t.ldb = nb; t.c = B(k, c); t.ldc = rows(k); t.side = 'A';
        dg_region_add(r, &t);
        mark_urgent(r);
      } else {
        t.op = DG_OP_TRSM; t.side = 'L'; t.uplo = uplo; t.transa = trans; t.diag = diag;
        t.m = rows(k); t.n = cols(c); t.alpha = 1.0; t.a = A(k, k); t.lda = rows(k);
        t.c = B(k, c); t.ldc = rows(k);
        dg_region_add(r, &t);
      }
      if (oz_ring && s + 1 < mt) {  // the solved block's columns, once per step
        memset(&t, 0, sizeof t);
        t.op = OP_OZ_SPLIT; t.trans = 'N'; t.a = B(k, c); t.lda = rows(k); t.m = rows(k);
        t.n = cols(c); t.c = xslot(step0 + s, c); t.ldc = ldk; t.k = nb;
        dg_region_add(r, &t);
        if (inv) mark_urgent(r);
      }
    }
    for (int s2 = s + 1; s2 < mt; s2++) {
      int m = forward ? s2 : mt - 1 - s2;
      int ai = (trans == 'N') ? m : k, aj = (trans == 'N') ? k : m;
      if (oz_ring) {
        // the rows of op(A(ai, aj)): rows of A(m, k) ('N'), columns of A(k, m) ('T')
        dg_task t;
        memset(&t, 0, sizeof t);
        t.op = OP_OZ_SPLIT; t.a = A(ai, aj); t.lda = rows(ai); t.m = rows(k); t.n = rows(m);
        t.trans = (trans == 'N') ? 'T' : 'N'; t.c = aslot(step0 + s, m); t.ldc = ldk; t.k = nb;
        dg_region_add(r, &t);
        for (int c = 0; c < bnt; c++) {
          memset(&t, 0, sizeof t);
          t.op = OP_OZ_GEMM; t.uplo = 'N'; t.m = rows(m); t.n = cols(c); t.k = rows(k);
          t.alpha = -1.0; t.beta = 1.0; t.a = aslot(step0 + s, m); t.b = xslot(step0 + s, c);
          t.lda = ldk; t.ldb = nb; t.c = B(m, c); t.ldc = rows(m);
          dg_region_add(r, &t);
          if (inv && s2 == s + 1) mark_urgent(r);  // the next diagonal block
        }
        continue;
      }
      for (int c = 0; c < bnt; c++) {
        dg_task t;
        memset(&t, 0, sizeof t);
        t.op = DG_OP_GEMM; t.transa = trans; t.transb = 'N'; t.m = rows(m); t.n = cols(c);
        t.k = rows(k); t.alpha = -1.0; t.beta = 1.0; t.a = A(ai, aj); t.lda = rows(ai);
        t.b = B(k, c); t.ldb = rows(k); t.c = B(m, c); t.ldc = rows(m);
        dg_region_add(r, &t);
      }
    }
  }
}

double *const *region_table(dg_region *r, const std::vector<double *> &ptrs) {
  r->tables.push_back(ptrs);
  return r->tables.back().data();
}

static size_t r256(size_t b) { return (b + 255) & ~(size_t)255; }

LuLayout lu_layout(int m, int n, int nb, bool pivot, bool emulated) {
  LuLayout L;
  const int mt = (m + nb - 1) / nb, nt = (n + nb - 1) / nb;
  const int steps = mt < nt ? mt : nt, mn = m < n ? m : n;
  size_t off = 256;
  L.leaf = off;
  off += r256(lu_leaf_scratch_bytes());
  L.lpiv = off;
  off += r256((size_t)mn * 4);
  L.list_cap = 2 * nb;
  L.list_stride = 1 + 2 * (size_t)L.list_cap;
  L.lists = off;
  off += r256((size_t)steps * L.list_stride * 4);
  if (pivot) {
    L.panel_bytes = r256((size_t)m * nb * 8);
    L.panel = off;
    off += 2 * L.panel_bytes;
  }
  if (emulated) {
    // the panel recursion's largest update: (rows) x (nb/2) x (nb/2 rounded up to 32)
    const int h = nb / 2 + 32;
    L.ozp_bytes = r256(oz_scratch_bytes(pivot ? m : nb, h, h, false));
    L.ozp = off;
    off += L.ozp_bytes;
    L.ring = off;
    off += (size_t)kOzRingDepth * (mt + nt) * oz_slot_bytes((nb + 7) / 8 * 8, nb);
    L.winv_bytes = r256((size_t)nb * nb * 8);
    L.winv = off;
    off += (size_t)kOzRingDepth * L.winv_bytes;
  }
  // the pivots as the region writes them; copied to the caller's ipiv after
  // the region, outside its graph (whose cache key then does not hold the
  // caller's buffer: a new ipiv per call replays the same graph)
  L.ipiv = off;
  off += r256((size_t)mn * 8);
  L.total = off;
  return L;
}

// lu.jl:306-410 (RowMaximum) / 5-54 (NoPivot).  Step k: the block column's
// tiles from the diagonal down are gathered into a panel buffer, factored
// (OP_LU_PANEL) and scattered back; its interchanges go to every other block
// column (swaprows_trail!, one task per block column); then TRSM('L', 'L',
// 'N', 'U') of the row panel and GEMM('N', 'N', -1) of the trailing tiles.
// Without pivoting the diagonal tile is factored in place and the column
// panel solved with TRSM('R', 'U', 'N', 'N').  With the emulated engine the
// rows of L(i, k) and the columns of U(k, j) are cut into slices once per
// step (ring slots (k mod depth, i) and (k mod depth, mt + j)) and every
// trailing tile takes one emulated product; each row panel tile is one
// emulated product with the inverse of L(k, k).
#ifndef DG_LU_GEMM_BLOCKS
#define DG_LU_GEMM_BLOCKS 3
#endif
// Output blocks per CTA of the LU's trailing updates (2..9; 1: one each).
// Three: a CTA forms one block's outputs while the tensor cores run the next,
// and still hands its SM back within about 0.15 ms to a leaf, which needs
// ~85 SMs at once (N = 32768: 874 ms against 897 with one block per CTA,
// 929 with six).
constexpr int kLuGemmBlocks = DG_LU_GEMM_BLOCKS;

void build_lu_region(dg_region *r, int m, int n, int nb, double *const *tiles, bool pivot,
                     void *ws, long long *ipiv, bool emulated) {
  const int mt = (m + nb - 1) / nb, nt = (n + nb - 1) / nb, steps = mt < nt ? mt : nt;
  auto rows = [&](int i) { return (i + 1) * nb <= m ? nb : m - i * nb; };
  auto cols = [&](int j) { return (j + 1) * nb <= n ? nb : n - j * nb; };
  auto T = [&](int i, int j) { return tiles[i + (size_t)j * mt]; };
  const LuLayout L = lu_layout(m, n, nb, pivot, emulated);
  char *w = (char *)ws;
  const int ldk = (nb + 7) / 8 * 8;
  const size_t sb = oz_slot_bytes(ldk, nb);
  const int slot_units = (int)(sb / 256);
  auto slot = [&](int k, int q) {
    return (double *)(w + L.ring + ((size_t)(k % kOzRingDepth) * (mt + nt) + q) * sb);
  };
  dg_task t;
  auto add = [&](int lvl) {
    dg_region_add(r, &t);
    mark_level(r, lvl);
  };
  for (int k = 0; k < steps; k++) {
    const int mk = m - k * nb, wk = cols(k);
    const int kk = rows(k) < wk ? rows(k) : wk;  // order of L(k, k) and U(k, k)
    double *P;
    int ldp;
    if (pivot) {
      P = (double *)(w + L.panel + (size_t)(k % 2) * L.panel_bytes);
      ldp = mk;
      for (int i = k; i < mt; i++) {
        memset(&t, 0, sizeof t);
        t.op = DG_OP_COPY; t.m = rows(i); t.n = wk; t.a = T(i, k); t.lda = rows(i);
        t.c = P + (size_t)(i - k) * nb; t.ldc = ldp;
        add(0);
      }
    } else {
      P = T(k, k);
      ldp = rows(k);
    }
    memset(&t, 0, sizeof t);
    t.op = OP_LU_PANEL; t.c = P; t.ldc = ldp; t.m = pivot ? mk : rows(k); t.n = wk;
    t.lda = m; t.k = n; t.ldb = nb; t.info_offset = k * nb; t.b = (const double *)ws;
    t.a = (const double *)ipiv; t.transa = pivot ? 'P' : 'N'; t.diag = emulated ? 'E' : 'N';
    add(0);
    if (pivot) {
      for (int i = k; i < mt; i++) {
        memset(&t, 0, sizeof t);
        t.op = DG_OP_COPY; t.m = rows(i); t.n = wk; t.a = P + (size_t)(i - k) * nb; t.lda = ldp;
        t.c = T(i, k); t.ldc = rows(i);
        add(0);
      }
      const int *lists = (const int *)(w + L.lists) + (size_t)k * L.list_stride;
      for (int j = 0; j < nt; j++) {
        if (j == k) continue;
        std::vector<double *> col;
        for (int i = k; i < mt; i++) col.push_back(T(i, j));
        memset(&t, 0, sizeof t);
        t.op = OP_LU_LASWP; t.a = (const double *)region_table(r, col); t.k = mt - k; t.m = mk;
        t.n = cols(j); t.ldb = nb; t.b = (const double *)lists; t.ldc = L.list_cap;
        add(j > k ? j - k - 1 : kPrioLevels - 1);
      }
    } else {
      for (int i = k + 1; i < mt; i++) {  // L(i, k) = A(i, k) U(k, k)^-1
        memset(&t, 0, sizeof t);
        t.op = emulated ? OP_OZ_TRSM : DG_OP_TRSM; t.side = 'R'; t.uplo = 'U'; t.transa = 'N';
        t.diag = 'N'; t.m = rows(i); t.n = kk; t.alpha = 1.0; t.a = T(k, k); t.lda = rows(k);
        t.c = T(i, k); t.ldc = rows(i);
        if (emulated) { t.b = slot(k, i); t.ldb = slot_units; }
        add(0);
      }
    }
    if (k + 1 >= nt) continue;
    // Emulated engine: the row panel's TRSMs become products with the inverse
    // W = L(k, k)^-1, formed once per step by substitution; W's rows go to
    // slot (k mod depth, k) with its unit diagonal kept apart (exact).
    double *Wk = (double *)(w + L.winv + (size_t)(k % kOzRingDepth) * L.winv_bytes);
    if (emulated) {
      memset(&t, 0, sizeof t);
      t.op = OP_LU_LINV; t.n = kk; t.a = T(k, k); t.lda = rows(k); t.c = Wk; t.ldc = kk;
      add(0);
      memset(&t, 0, sizeof t);
      t.op = OP_OZ_SPLIT; t.a = Wk; t.lda = kk; t.m = kk; t.n = kk; t.trans = 'T'; t.diag = 'Z';
      t.c = slot(k, k); t.ldc = ldk; t.k = nb;
      add(0);
    }
    if (emulated)
      for (int i = k + 1; i < mt; i++) {  // the rows of L(i, k): A-vectors of length kk
        memset(&t, 0, sizeof t);
        t.op = OP_OZ_SPLIT; t.trans = 'T'; t.a = T(i, k); t.lda = rows(i); t.m = kk;
        t.n = rows(i); t.c = slot(k, i); t.ldc = ldk; t.k = nb;
        add(0);
      }
    for (int j = k + 1; j < nt; j++) {
      const int lvl = j - k - 1;
      if (emulated) {  // U(k, j) = W A(k, j) = A(k, j) + offdiag(W) A(k, j)
        memset(&t, 0, sizeof t);
        t.op = OP_OZ_SPLIT; t.trans = 'N'; t.a = T(k, j); t.lda = rows(k); t.m = kk;
        t.n = cols(j); t.c = slot(k, mt + j); t.ldc = ldk; t.k = nb;
        add(lvl);
        memset(&t, 0, sizeof t);
        t.op = OP_OZ_GEMM; t.uplo = 'N'; t.m = kk; t.n = cols(j); t.k = kk; t.alpha = 1.0;
        t.beta = 0.0; t.a = slot(k, k); t.b = slot(k, mt + j); t.lda = ldk; t.ldb = nb;
        t.c = T(k, j); t.ldc = rows(k); t.side = 'A';
        add(lvl);
      } else {  // U(k, j) = L(k, k)^-1 A(k, j)
        memset(&t, 0, sizeof t);
        t.op = DG_OP_TRSM; t.side = 'L'; t.uplo = 'L'; t.transa = 'N'; t.diag = 'U';
        t.m = kk; t.n = cols(j); t.alpha = 1.0; t.a = T(k, k); t.lda = rows(k);
        t.c = T(k, j); t.ldc = rows(k);
        add(lvl);
      }
      if (k + 1 >= mt) continue;
      if (emulated) {  // the columns of U(k, j): B-vectors of length kk
        memset(&t, 0, sizeof t);
        t.op = OP_OZ_SPLIT; t.trans = 'N'; t.a = T(k, j); t.lda = rows(k); t.m = kk;
        t.n = cols(j); t.c = slot(k, mt + j); t.ldc = ldk; t.k = nb;
        add(lvl);
      }
      for (int i = k + 1; i < mt; i++) {  // A(i, j) -= L(i, k) U(k, j)
        memset(&t, 0, sizeof t);
        if (emulated) {
          // a few output blocks per CTA (kLuGemmBlocks): short CTAs hand their
          // SMs back soon to the panel's leaves, which need many SMs at once
          t.op = OP_OZ_GEMM; t.uplo = 'N'; t.m = rows(i); t.n = cols(j); t.k = kk;
          t.alpha = -1.0; t.beta = 1.0; t.a = slot(k, i); t.b = slot(k, mt + j);
          t.lda = ldk; t.ldb = nb; t.c = T(i, j); t.ldc = rows(i);
          if (kLuGemmBlocks > 1) t.diag = (char)('0' + kLuGemmBlocks);
        } else {
          t.op = DG_OP_GEMM; t.transa = 'N'; t.transb = 'N'; t.m = rows(i); t.n = cols(j);
          t.k = kk; t.alpha = -1.0; t.beta = 1.0; t.a = T(i, k); t.lda = rows(i);
          t.b = T(k, j); t.ldb = rows(k); t.c = T(i, j); t.ldc = rows(i);
        }
        add(lvl);
      }
    }
  }
}

size_t lu_solve_bytes(int n, int nb, int nrhs, bool emulated) {
  const int bnt = (nrhs + nb - 1) / nb;
  size_t b = emulated ? r256(oz_solve_ring_bytes_for(n, nb, nrhs)) : 0;
  b += r256((size_t)n * 4);
  for (int c = 0; c < bnt; c++) {
    const int w = (c + 1) * nb <= nrhs ? nb : nrhs - c * nb;
    b += r256((size_t)n * w * 8);
  }
  return b + r256((size_t)n * 8);  // the pivots, copied in before the region
}

size_t lu_solve_ipiv_offset(int n, int nb, int nrhs, bool emulated) {
  return lu_solve_bytes(n, nb, nrhs, emulated) - r256((size_t)n * 8);
}

// linalg.jl:264-308: B's rows permuted by the pivots (one permutation
// applied per block column of B), then ldiv!(UnitLowerTriangular) and
// ldiv!(UpperTriangular) as the two block solve passes.
void build_lu_solve_region(dg_region *r, int n, int nb, double *const *tiles,
                           const long long *ipiv, int nrhs, double *const *btiles, void *ws,
                           bool emulated) {
  const int mt = (n + nb - 1) / nb, bnt = (nrhs + nb - 1) / nb;
  char *w = (char *)ws;
  void *ring = emulated ? w : nullptr;
  size_t off = emulated ? r256(oz_solve_ring_bytes_for(n, nb, nrhs)) : 0;
  int *perm = (int *)(w + off);
  off += r256((size_t)n * 4);
  dg_task t;
  memset(&t, 0, sizeof t);
  t.op = OP_LU_PERM; t.a = (const double *)ipiv; t.k = n; t.n = n; t.c = (double *)perm;
  dg_region_add(r, &t);
  mark_urgent(r);
  for (int c = 0; c < bnt; c++) {
    const int wc = (c + 1) * nb <= nrhs ? nb : nrhs - c * nb;
    std::vector<double *> col;
    for (int i = 0; i < mt; i++) col.push_back(btiles[i + (size_t)c * mt]);
    memset(&t, 0, sizeof t);
    t.op = OP_LU_ROWS; t.a = (const double *)region_table(r, col); t.k = mt; t.m = n; t.n = wc;
    t.ldb = nb; t.b = (const double *)perm; t.c = (double *)(w + off);
    dg_region_add(r, &t);
    mark_urgent(r);
    off += r256((size_t)n * wc * 8);
  }
  build_solve_pass(r, 'L', 'N', n, nb, tiles, nrhs, btiles, ring, 0, nullptr, 'U');
  build_solve_pass(r, 'U', 'N', n, nb, tiles, nrhs, btiles, ring, mt, nullptr, 'N');
}

}  // namespace dg

namespace {
// The arguments that decide a whole-call region, zero-padded for hashing.
struct CallArgs {
  int64_t n, nb, nrhs, ldh;
  const void *ring, *winv, *host;
  char uplo;
};
uint64_t call_key(int fn, char uplo, int n, int nb, int nrhs, long long ldh, const void *ring,
                  const void *winv, const void *host, double *const *tiles,
                  double *const *btiles) {
  CallArgs a;
  memset(&a, 0, sizeof a);
  a.n = n; a.nb = nb; a.nrhs = nrhs; a.ldh = ldh;
  a.ring = ring; a.winv = winv; a.host = host; a.uplo = uplo;
  const size_t mt = (size_t)(n + nb - 1) / nb;
  uint64_t h = dg::call_hash(fn, &a, sizeof a, (const void *const *)tiles, mt * mt);
  if (btiles) {
    const size_t bnt = (size_t)(nrhs + nb - 1) / nb;
    h = dg::call_hash(fn, &h, sizeof h, (const void *const *)btiles, mt * bnt);
  }
  return h;
}
}  // namespace

// C = beta C over a tile grid (the empty contraction).
static int scale_tiles(int m, int n, int nb, double beta, double *const *C, cudaStream_t s) {
  const int mt = (m + nb - 1) / nb, nt = (n + nb - 1) / nb;
  for (int j = 0; j < nt; j++)
    for (int i = 0; i < mt; i++) {
      const int r = (i + 1) * nb <= m ? nb : m - i * nb, c = (j + 1) * nb <= n ? nb : n - j * nb;
      DG_TRY(dg::scale_f64(r, c, beta, C[i + (size_t)j * mt], r, nullptr, s));
    }
  return 0;
}

extern "C" int dg_gemm_tiled(char transa, char transb, int m, int n, int k, int nb, double alpha,
                             double *const *atiles, double *const *btiles, double beta,
                             double *const *ctiles, void *stream) {
  DG_CHECK_ARG(is_one_of(transa, "NnTtCc"), 1);
  DG_CHECK_ARG(is_one_of(transb, "NnTtCc"), 2);
  DG_CHECK_ARG(m >= 0, 3);
  DG_CHECK_ARG(n >= 0, 4);
  DG_CHECK_ARG(k >= 0, 5);
  DG_CHECK_ARG(nb > 0, 6);
  if (m == 0 || n == 0) return 0;
  DG_CHECK_ARG(ctiles != nullptr, 11);
  if (k == 0 || alpha == 0.0) return scale_tiles(m, n, nb, beta, ctiles, (cudaStream_t)stream);
  DG_CHECK_ARG(atiles != nullptr, 8);
  DG_CHECK_ARG(btiles != nullptr, 9);
  const char ta = is_one_of(transa, "Nn") ? 'N' : 'T', tb = is_one_of(transb, "Nn") ? 'N' : 'T';
  dg::WsLease lease;
  void *ring = nullptr;
  if (dg::get_f64_engine() == 2 && nb <= 1024)
    DG_TRY(lease.acquire(dg::mul_ring_bytes_for(m, n, nb), (cudaStream_t)stream, &ring));
  const size_t mt = (m + nb - 1) / nb, nt = (n + nb - 1) / nb, kt = (k + nb - 1) / nb;
  struct { int64_t m, n, k, nb; double alpha, beta; const void *ring; char ta, tb; } a;
  memset(&a, 0, sizeof a);
  a.m = m; a.n = n; a.k = k; a.nb = nb; a.alpha = alpha; a.beta = beta; a.ring = ring;
  a.ta = ta; a.tb = tb;
  uint64_t key = dg::call_hash(6, &a, sizeof a, (const void *const *)atiles, mt * kt);
  key = dg::call_hash(6, &key, sizeof key, (const void *const *)btiles, kt * nt);
  key = dg::call_hash(6, &key, sizeof key, (const void *const *)ctiles, mt * nt);
  return dg::region_run_cached(
      key,
      [&](dg_region *r) {
        dg::build_gemm_region(r, ta, tb, m, n, k, nb, alpha, atiles, btiles, beta, ctiles, ring);
      },
      (cudaStream_t)stream, true);
}

extern "C" int dg_syrk_tiled(char trans, int n, int k, int nb, double alpha,
                             double *const *atiles, double beta, double *const *ctiles,
                             void *stream) {
  DG_CHECK_ARG(is_one_of(trans, "NnTtCc"), 1);
  DG_CHECK_ARG(n >= 0, 2);
  DG_CHECK_ARG(k >= 0, 3);
  DG_CHECK_ARG(nb > 0, 4);
  if (n == 0) return 0;
  DG_CHECK_ARG(ctiles != nullptr, 8);
  const char tr = is_one_of(trans, "Nn") ? 'N' : 'T';
  const size_t nt = (n + nb - 1) / nb, kt = (k + nb - 1) / nb;
  if (k == 0 || alpha == 0.0) {
    DG_TRY(scale_tiles(n, n, nb, beta, ctiles, (cudaStream_t)stream));
    return dg::region_run_cached(
        dg::call_hash(8, &nb, sizeof nb, (const void *const *)ctiles, nt * nt),
        [&](dg_region *r) {
          const int nn = n;
          dg::build_syrk_region(r, tr, nn, 0, nb, 0.0, nullptr, 1.0, ctiles, nullptr);
        },
        (cudaStream_t)stream, true);
  }
  DG_CHECK_ARG(atiles != nullptr, 6);
  dg::WsLease lease;
  void *ring = nullptr;
  if (dg::get_f64_engine() == 2 && nb <= 1024)
    DG_TRY(lease.acquire(dg::mul_ring_bytes_for(n, 0, nb), (cudaStream_t)stream, &ring));
  struct { int64_t n, k, nb; double alpha, beta; const void *ring; char tr; } a;
  memset(&a, 0, sizeof a);
  a.n = n; a.k = k; a.nb = nb; a.alpha = alpha; a.beta = beta; a.ring = ring; a.tr = tr;
  uint64_t key = dg::call_hash(7, &a, sizeof a, (const void *const *)atiles, nt * kt);
  key = dg::call_hash(7, &key, sizeof key, (const void *const *)ctiles, nt * nt);
  return dg::region_run_cached(
      key,
      [&](dg_region *r) {
        dg::build_syrk_region(r, tr, n, k, nb, alpha, atiles, beta, ctiles, ring);
      },
      (cudaStream_t)stream, true);
}

extern "C" int dg_cholesky_tiled(char uplo, int n, int nb, double *const *tiles, void *stream) {
  DG_CHECK_ARG(is_one_of(uplo, "ULul"), 1);
  DG_CHECK_ARG(n >= 0, 2);
  DG_CHECK_ARG(nb > 0, 3);
  DG_CHECK_ARG(tiles != nullptr || n == 0, 4);
  if (n == 0) return 0;
  dg::WsLease lease;
  void *ring = nullptr;
  if (dg::get_f64_engine() == 2 && nb <= 1024)
    DG_TRY(lease.acquire(dg::oz_ring_bytes_for(n, nb), (cudaStream_t)stream, &ring));
  return dg::region_run_cached(
      call_key(1, uplo, n, nb, 0, 0, ring, nullptr, nullptr, tiles, nullptr),
      [&](dg_region *r) { dg::build_cholesky_region(r, uplo, n, nb, tiles, ring); },
      (cudaStream_t)stream, true);
}

// The kept inverses of the diagonal tiles are formed in the stream's
// workspace, after the slice slots, and copied to the caller's winv once the
// region has run: the region's graph then holds only workspace addresses, so
// a new winv buffer per call replays the cached graph (mt nb^2 doubles, about
// 0.1 ms of copy at N = 32768).
static size_t winv_ring_bytes(int n, int nb) {
  const size_t mt = (size_t)((n + nb - 1) / nb);
  return ((dg::oz_ring_bytes_for(n, nb) + 255) & ~(size_t)255) + mt * nb * nb * 8;
}
static double *winv_in_ring(void *ring, int n, int nb) {
  return (double *)((char *)ring + ((dg::oz_ring_bytes_for(n, nb) + 255) & ~(size_t)255));
}
static int winv_copy_out(double *winv, const double *wws, int n, int nb, cudaStream_t s) {
  const size_t mt = (size_t)((n + nb - 1) / nb);
  DG_CUDA_TRY(cudaMemcpyAsync(winv, wws, mt * nb * nb * 8, cudaMemcpyDeviceToDevice, s));
  DG_CUDA_TRY(cudaStreamSynchronize(s));
  return 0;
}

extern "C" int dg_cholesky_tiled_winv(char uplo, int n, int nb, double *const *tiles,
                                      double *winv, void *stream) {
  DG_CHECK_ARG(is_one_of(uplo, "ULul"), 1);
  DG_CHECK_ARG(n >= 0, 2);
  DG_CHECK_ARG(nb > 0, 3);
  DG_CHECK_ARG(tiles != nullptr || n == 0, 4);
  DG_CHECK_ARG(winv != nullptr || n == 0, 5);
  if (dg::get_f64_engine() != 2 || nb > 1024) return DG_ERR_UNSUPPORTED;
  if (n == 0) return 0;
  dg::WsLease lease;
  void *ring = nullptr;
  DG_TRY(lease.acquire(winv_ring_bytes(n, nb), (cudaStream_t)stream, &ring));
  double *wws = winv_in_ring(ring, n, nb);
  const int rc = dg::region_run_cached(
      call_key(2, uplo, n, nb, 0, 0, ring, wws, nullptr, tiles, nullptr),
      [&](dg_region *r) { dg::build_cholesky_region(r, uplo, n, nb, tiles, ring, wws); },
      (cudaStream_t)stream, true);
  if (rc < 0) return rc;
  DG_TRY(winv_copy_out(winv, wws, n, nb, (cudaStream_t)stream));
  return rc;
}

extern "C" int dg_cholesky_tiled_host(char uplo, int n, int nb, const double *host,
                                      long long ldh, double *const *tiles, double *winv,
                                      void *stream) {
  DG_CHECK_ARG(is_one_of(uplo, "ULul"), 1);
  DG_CHECK_ARG(n >= 0, 2);
  DG_CHECK_ARG(nb > 0, 3);
  if (n == 0) return 0;
  DG_CHECK_ARG(ldh >= n && ldh <= 2147483647LL, 5);
  // the kernels read the source directly: page-locked host or device memory
  DG_CHECK_ARG(host != nullptr && dg::device_readable(host) &&
                   dg::device_readable(host + (size_t)(n - 1) * ldh + (n - 1)),
               4);
  DG_CHECK_ARG(tiles != nullptr, 6);
  const bool emulated = dg::get_f64_engine() == 2 && nb <= 1024;
  if (winv && !emulated) return DG_ERR_UNSUPPORTED;
  dg::WsLease lease;
  void *ring = nullptr;
  if (emulated)
    DG_TRY(lease.acquire(winv ? winv_ring_bytes(n, nb) : dg::oz_ring_bytes_for(n, nb),
                         (cudaStream_t)stream, &ring));
  double *wws = winv ? winv_in_ring(ring, n, nb) : nullptr;
  const int rc = dg::region_run_cached(
      call_key(3, uplo, n, nb, 0, ldh, ring, wws, host, tiles, nullptr),
      [&](dg_region *r) {
        dg::build_upload_tasks(r, uplo, n, nb, tiles, host, ldh);
        dg::build_cholesky_region(r, uplo, n, nb, tiles, ring, wws);
      },
      (cudaStream_t)stream, true);
  if (rc < 0 || !winv) return rc;
  DG_TRY(winv_copy_out(winv, wws, n, nb, (cudaStream_t)stream));
  return rc;
}

extern "C" int dg_cholesky_solve_tiled_winv(char uplo, int n, int nb, double *const *tiles,
                                            const double *winv, int nrhs,
                                            double *const *btiles, void *stream) {
  DG_CHECK_ARG(is_one_of(uplo, "ULul"), 1);
  DG_CHECK_ARG(n >= 0, 2);
  DG_CHECK_ARG(nb > 0, 3);
  DG_CHECK_ARG(nrhs >= 0, 6);
  if (dg::get_f64_engine() != 2 || nb > 1024) return DG_ERR_UNSUPPORTED;
  if (n == 0 || nrhs == 0) return 0;
  DG_CHECK_ARG(tiles != nullptr, 4);
  DG_CHECK_ARG(winv != nullptr, 5);
  DG_CHECK_ARG(btiles != nullptr, 7);
  const bool up = (uplo == 'U' || uplo == 'u');
  dg::WsLease lease;
  void *ring = nullptr;
  DG_TRY(lease.acquire(dg::oz_solve_ring_bytes_for(n, nb, nrhs, true), (cudaStream_t)stream,
                       &ring));
  const int mt = (n + nb - 1) / nb;
  return dg::region_run_cached(
      call_key(4, uplo, n, nb, nrhs, 0, ring, winv, nullptr, tiles, btiles),
      [&](dg_region *r) {
        dg::build_solve_pass(r, up ? 'U' : 'L', up ? 'T' : 'N', n, nb, tiles, nrhs, btiles, ring,
                             0, winv);
        dg::build_solve_pass(r, up ? 'U' : 'L', up ? 'N' : 'T', n, nb, tiles, nrhs, btiles, ring,
                             mt, winv);
      },
      (cudaStream_t)stream, true);
}

extern "C" int dg_cholesky_solve_tiled(char uplo, int n, int nb, double *const *tiles, int nrhs,
                                       double *const *btiles, void *stream) {
  DG_CHECK_ARG(is_one_of(uplo, "ULul"), 1);
  DG_CHECK_ARG(n >= 0, 2);
  DG_CHECK_ARG(nb > 0, 3);
  DG_CHECK_ARG(nrhs >= 0, 5);
  if (n == 0 || nrhs == 0) return 0;
  DG_CHECK_ARG(tiles != nullptr, 4);
  DG_CHECK_ARG(btiles != nullptr, 6);
  const bool up = (uplo == 'U' || uplo == 'u');
  dg::WsLease lease;
  void *ring = nullptr;
  if (dg::get_f64_engine() == 2 && nb <= 1024)
    DG_TRY(lease.acquire(dg::oz_solve_ring_bytes_for(n, nb, nrhs), (cudaStream_t)stream, &ring));
  const int mt = (n + nb - 1) / nb;
  return dg::region_run_cached(
      call_key(5, uplo, n, nb, nrhs, 0, ring, nullptr, nullptr, tiles, btiles),
      [&](dg_region *r) {
        dg::build_solve_pass(r, up ? 'U' : 'L', up ? 'T' : 'N', n, nb, tiles, nrhs, btiles, ring, 0);
        dg::build_solve_pass(r, up ? 'U' : 'L', up ? 'N' : 'T', n, nb, tiles, nrhs, btiles, ring, mt);
      },
      (cudaStream_t)stream, true);
}

// ---------------------------------------------------------------------------
// Tiled LU (src/array/lu.jl, linalg.jl:264-308).
// ---------------------------------------------------------------------------
namespace {
constexpr int kLuNoInfo = 0x7f7f7f7f;  // the info word before a zero pivot lowers it

struct LuCallArgs {
  int64_t m, n, nb, nrhs, pivot, emulated;
  const void *ws, *ipiv;
};

uint64_t lu_key(int fn, int64_t m, int64_t n, int64_t nb, int64_t nrhs, int64_t pivot,
                int64_t emulated, const void *ws, const void *ipiv, double *const *tiles,
                size_t ntiles, double *const *btiles, size_t nbtiles) {
  LuCallArgs a;
  memset(&a, 0, sizeof a);
  a.m = m; a.n = n; a.nb = nb; a.nrhs = nrhs; a.pivot = pivot; a.emulated = emulated;
  a.ws = ws; a.ipiv = ipiv;
  uint64_t h = dg::call_hash(fn, &a, sizeof a, (const void *const *)tiles, ntiles);
  if (btiles) h = dg::call_hash(fn, &h, sizeof h, (const void *const *)btiles, nbtiles);
  return h;
}

// The status word (a timed-out wait) and the info word after the work queued
// on s: DG_ERR_TIMEOUT, else the first zero pivot's column (1-based) or 0.
int lu_words_reset(void *ws, cudaStream_t s) {
  DG_CUDA_TRY(cudaMemsetAsync(ws, 0, 4, s));
  DG_CUDA_TRY(cudaMemsetAsync((char *)ws + 4, 0x7f, 4, s));
  return 0;
}
int lu_words_read(const void *ws, cudaStream_t s) {
  int v[2] = {0, 0};
  DG_CUDA_TRY(cudaMemcpyAsync(v, ws, sizeof v, cudaMemcpyDeviceToHost, s));
  DG_CUDA_TRY(cudaStreamSynchronize(s));
  if (v[0]) return DG_ERR_TIMEOUT;
  return v[1] == kLuNoInfo ? 0 : v[1];
}
}  // namespace

extern "C" int dg_getrf(int m, int n, double *A, int lda, long long *ipiv, int *info_host,
                        void *stream) {
  DG_CHECK_ARG(m >= 0, 1);
  DG_CHECK_ARG(n >= 0, 2);
  DG_CHECK_ARG(lda >= (m > 1 ? m : 1), 4);
  DG_CHECK_ARG(info_host != nullptr, 6);
  *info_host = 0;
  if (m == 0 || n == 0) return 0;
  DG_CHECK_ARG(A != nullptr, 3);
  DG_CHECK_ARG(ipiv != nullptr, 5);
  const bool emulated = dg::get_f64_engine() == 2;
  auto r256 = [](size_t b) { return (b + 255) & ~(size_t)255; };
  const size_t leaf = r256(dg::lu_leaf_scratch_bytes());
  const size_t lpiv = r256((size_t)(m < n ? m : n) * 4);
  const int h = n / 2 + 32;
  const size_t ozp = emulated ? r256(dg::oz_scratch_bytes(m, h, h, false)) : 0;
  dg::lu_prepare();
  dg::WsLease lease;
  void *ws = nullptr;
  DG_TRY(lease.acquire(256 + leaf + lpiv + ozp, (cudaStream_t)stream, &ws));
  char *w = (char *)ws;
  cudaStream_t s = (cudaStream_t)stream;
  DG_TRY(lu_words_reset(ws, s));
  DG_TRY(dg::lu_panel_f64(A, lda, m, n, true, (int *)(w + 256 + leaf), (int *)(w + 4), 0,
                          w + 256, (int *)w, ozp ? w + 256 + leaf + lpiv : nullptr, ozp, ipiv,
                          nullptr, 0, s));
  const int rc = lu_words_read(ws, s);
  if (rc >= 0) *info_host = rc;
  return rc;
}

constexpr int kLuStreams = 4;

extern "C" int dg_lu_tiled(int m, int n, int nb, double *const *tiles, int pivot,
                           long long *ipiv, void *stream) {
  DG_CHECK_ARG(m >= 0, 1);
  DG_CHECK_ARG(n >= 0, 2);
  DG_CHECK_ARG(nb > 0, 3);
  DG_CHECK_ARG(pivot == 0 || pivot == 1, 5);
  if (m == 0 || n == 0) return 0;
  DG_CHECK_ARG(tiles != nullptr, 4);
  DG_CHECK_ARG(ipiv != nullptr, 6);
  const int mt = (m + nb - 1) / nb, nt = (n + nb - 1) / nb;
  if (nb > 1024 || mt > dg::kMaxTileRows) return DG_ERR_UNSUPPORTED;
  const bool emulated = dg::get_f64_engine() == 2;
  const dg::LuLayout L = dg::lu_layout(m, n, nb, pivot != 0, emulated);
  dg::lu_prepare();
  dg::WsLease lease;
  void *ws = nullptr;
  DG_TRY(lease.acquire(L.total, (cudaStream_t)stream, &ws));
  cudaStream_t s = (cudaStream_t)stream;
  DG_TRY(lu_words_reset(ws, s));
  long long *wpiv = (long long *)((char *)ws + L.ipiv);
  // Four streams at the lowest priority (two per level above): the LU's
  // trailing updates are few large launches per step, and fewer concurrent
  // streams let the cooperative leaf launches, which need ~85 SMs at once,
  // start sooner (N = 32768: 832 ms against 874 with sixteen).
  const int rc = dg::region_run_cached(
      lu_key(30, m, n, nb, 0, pivot, emulated, ws, nullptr, tiles, (size_t)mt * nt, nullptr, 0),
      [&](dg_region *r) { dg::build_lu_region(r, m, n, nb, tiles, pivot != 0, ws, wpiv, emulated); },
      s, true, kLuStreams);
  if (rc) return rc;
  const int mn = m < n ? m : n;
  if (pivot)
    DG_CUDA_TRY(cudaMemcpyAsync(ipiv, wpiv, sizeof(long long) * (size_t)mn,
                                cudaMemcpyDeviceToDevice, s));
  else
    DG_TRY(dg::lu_iota(ipiv, mn, s));
  return lu_words_read(ws, s);
}

extern "C" int dg_lu_solve_tiled(int n, int nb, double *const *tiles, const long long *ipiv,
                                 int nrhs, double *const *btiles, void *stream) {
  DG_CHECK_ARG(n >= 0, 1);
  DG_CHECK_ARG(nb > 0, 2);
  DG_CHECK_ARG(nrhs >= 0, 5);
  if (n == 0 || nrhs == 0) return 0;
  DG_CHECK_ARG(tiles != nullptr, 3);
  DG_CHECK_ARG(ipiv != nullptr, 4);
  DG_CHECK_ARG(btiles != nullptr, 6);
  const int mt = (n + nb - 1) / nb, bnt = (nrhs + nb - 1) / nb;
  if (mt > dg::kMaxTileRows) return DG_ERR_UNSUPPORTED;
  const bool emulated = dg::get_f64_engine() == 2 && nb <= 1024;
  dg::lu_prepare();
  dg::WsLease lease;
  void *ws = nullptr;
  DG_TRY(lease.acquire(dg::lu_solve_bytes(n, nb, nrhs, emulated), (cudaStream_t)stream, &ws));
  // the pivots enter through the workspace, so that the graph does not hold
  // the caller's ipiv buffer
  long long *wpiv =
      (long long *)((char *)ws + dg::lu_solve_ipiv_offset(n, nb, nrhs, emulated));
  DG_CUDA_TRY(cudaMemcpyAsync(wpiv, ipiv, sizeof(long long) * (size_t)n,
                              cudaMemcpyDeviceToDevice, (cudaStream_t)stream));
  return dg::region_run_cached(
      lu_key(31, n, n, nb, nrhs, 1, emulated, ws, nullptr, tiles, (size_t)mt * mt, btiles,
             (size_t)mt * bnt),
      [&](dg_region *r) {
        dg::build_lu_solve_region(r, n, nb, tiles, wpiv, nrhs, btiles, ws, emulated);
      },
      (cudaStream_t)stream, true);
}
