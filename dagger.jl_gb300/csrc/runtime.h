// Internal host-runtime declarations shared by the translation units of
// libdaggergb300 (not part of the public ABI).
#pragma once

#include <cuda_runtime.h>

#include <map>
#include <memory>
#include <mutex>
#include <functional>
#include <vector>

#include "../../include/dagger_gb300.h"

namespace dg {

#ifndef DG_REGION_STREAMS
#define DG_REGION_STREAMS 16
#endif
constexpr int kDefaultStreams = DG_REGION_STREAMS;
#ifndef DG_URGENT_STREAMS
#define DG_URGENT_STREAMS 4
#endif
constexpr int kUrgentStreams = DG_URGENT_STREAMS;  // streams per priority level above the lowest
constexpr int kPrioLevels = 6;     // stream priority levels used (fewer on the device collapse)
// Host-to-device uploads get their own class of streams (at the least
// priority), so that no compute task queues behind a transfer it does not need.
constexpr int kTransferLevel = kPrioLevels, kTransferStreams = 4;

// Internal task kinds of the tiled Cholesky region with the emulated FP64
// engine (not part of the public dg_op enumeration):
//   OP_OZ_SPLIT  a = FP64 tile (lda), m = vector length K, n = vectors,
//                trans 'N' = the tile's columns, 'T' = its rows; c = slice slot,
//                ldc = ldk, k = slot capacity in vectors
//   OP_OZ_GEMM   a, b = slice slots (lda = ldk, ldb = slot capacity), c = FP64
//                tile (ldc), m x n output, k = K, alpha, beta; uplo 'U' / 'L'
//                stores one triangle; diag 'P' (off the critical path): each
//                CTA computes kOzBlocksPerCta output blocks in turn; diag
//                '2'..'9': that many blocks per CTA
//   OP_OZ_TRSM   DG_OP_TRSM whose recursion updates are emulated, with
//   OP_OZ_POTRF  (likewise DG_OP_POTRF) b = slice scratch of ldb * 256 bytes
//   OP_OZ_ZERO   c (m x n, ldc) = 0
//   OP_UPLOAD    c (m x n tile, ldc = m) = the row-major block at a (row
//                stride lda) in page-locked host or device memory
//   OP_TILE_T    c (n x m, ldc) = a (m x n, lda)'
//   OP_TILE_MIRROR  c (n x n, ldc): the upper triangle copied to the lower
//   OP_OZ_INV    c (n x n, ldc) = U^-T for uplo 'U' / L^-T for 'L' of the
//                factor tile a (lda), by substitution on the identity; b, ldb
//                slice scratch as above
constexpr int OP_OZ_SPLIT = 100;
constexpr int OP_OZ_GEMM = 101;
constexpr int OP_OZ_TRSM = 102;
constexpr int OP_OZ_POTRF = 103;
constexpr int OP_OZ_INV = 104;
constexpr int OP_OZ_ZERO = 105;
constexpr int OP_UPLOAD = 106;
constexpr int OP_TILE_T = 107;
constexpr int OP_TILE_MIRROR = 108;
// Tiled LU (lu.cu):
//   OP_LU_PANEL  the m x n panel c (ldc) factored in place, transa 'P' with
//                row interchanges, 'N' without; diag 'E': emulated updates;
//                lda x k = the whole matrix, ldb = nb, info_offset = the
//                panel's first row; b = the LU workspace (lu_layout), a = ipiv
//   OP_LU_LASWP  a panel's row list (b, int, ldc = its capacity) applied to
//                a block column: a = host array of its k tile pointers (m rows
//                in all, ldb = nb per tile), n columns
//   OP_LU_PERM   c (int, n) = the composite of k interchanges a (int64 ipiv)
//   OP_LU_ROWS   a block column of k tiles (a = host array of tile pointers,
//                m rows, n columns, ldb = nb) permuted by b (OP_LU_PERM's
//                result) through c (m x n doubles)
constexpr int OP_LU_PANEL = 109;
constexpr int OP_LU_LASWP = 110;
constexpr int OP_LU_PERM = 111;
constexpr int OP_LU_ROWS = 112;
//   OP_LU_LINV   c (n x n, ldc) = L^-1 of the unit lower triangle of a (lda)
constexpr int OP_LU_LINV = 113;
constexpr int kOpLast = OP_LU_LINV;
constexpr int kOzRingDepth = 3;  // steps whose slices can be live at once
#ifndef DG_OZ_BLOCKS_PER_CTA
#define DG_OZ_BLOCKS_PER_CTA 6
#endif
constexpr int kOzBlocksPerCta = DG_OZ_BLOCKS_PER_CTA;
size_t oz_slot_bytes(long long ldk, long long cap);
size_t oz_ring_bytes_for(int n, int nb);

// The emulated FP64 engine's and the LU's workspace (slice slots, leaf
// scratch, pivot words) of one stream.  Calls issued on different streams
// use different workspaces and run concurrently; calls on the same stream
// handle take turns through a lease (below).
struct Workspace {
  std::mutex use;               // held by the lease from acquisition to release
  void *p = nullptr;            // stream-ordered allocation of the library pool
  size_t bytes = 0;
  cudaEvent_t done = nullptr;   // recorded on the stream when a lease ends
  bool recorded = false;
};

// Library-owned per-device state.
struct DeviceState {
  static constexpr int kInfoWords = 4096;
  std::mutex mu;
  int *info_words = nullptr;  // ring of device ints for synchronous calls
  unsigned next_info = 0;
  int scratch_int(int **p);
  std::map<cudaStream_t, std::unique_ptr<Workspace>> workspaces;  // by stream handle
  Workspace *workspace_of(cudaStream_t s);
  // Frees the workspaces no lease holds, once the work queued with them is
  // done (dg_release_memory).
  void release_idle_workspaces();
  ~DeviceState();
};

// Exclusive use of the calling stream's workspace, grown to `bytes`, from
// acquire() until the lease goes out of scope.  acquire() blocks while
// another host thread holds a lease on the same stream handle, then makes the
// stream wait for the work the previous lease queued; growth frees the old
// block and allocates the new one in stream order (no device-wide
// synchronisation, so calls on other streams keep running).  The release
// records the workspace's event on the stream after everything the call
// queued.  Graph and call caches key on the workspace address, so a graph
// built for one stream's workspace is never launched with another's.
class WsLease {
 public:
  WsLease() = default;
  WsLease(const WsLease &) = delete;
  WsLease &operator=(const WsLease &) = delete;
  ~WsLease();
  int acquire(size_t bytes, cudaStream_t s, void **p);

 private:
  Workspace *w_ = nullptr;
  cudaStream_t s_ = nullptr;
};

DeviceState &device_state();
std::vector<cudaStream_t> &stream_pool(int want, int level = kPrioLevels - 1);
// The priority level of the last task added: 0 = on the critical path, up to
// kPrioLevels - 1 (the default) for work needed last.
void mark_level(dg_region *r, int level);
void mark_urgent(dg_region *r);  // mark_level(r, 0)
void mark_transfer(dg_region *r);  // the last task added is an upload

// Strided byte footprint of a column-major matrix argument.
struct Footprint {
  uintptr_t base = 0, lo = 0, hi = 0;
  int64_t rows = 0, cols = 0, ld = 1;  // rows and ld in bytes
};
Footprint footprint(const void *p, int rows, int cols, int ld, int elem);
bool overlaps(const Footprint &a, const Footprint &b);

int run_task(const dg_task &t, int *info, cudaStream_t s);
int region_run(dg_region *r, int use_graph, int serial, cudaStream_t origin, int stream_pool_size,
               bool sync);
void clear_graphs();
// A whole-call region: `call` hashes the entry point's arguments
// (call_hash); when a graph for the same call is cached it is launched
// without building the region, else build(r) fills a region that is run and
// remembered on `streams` streams at the lowest priority.  The f64 engine,
// the device and the stream count join the key.
int region_run_cached(uint64_t call, const std::function<void(dg_region *)> &build,
                      cudaStream_t origin, bool sync, int streams = kDefaultStreams);
uint64_t call_hash(int fn, const void *args, size_t bytes, const void *const *ptrs, size_t nptrs);

// oz_ring != nullptr selects the emulated-FP64 trailing updates, with
// oz_ring_bytes_for(n, nb) bytes of slice slots (nb <= 1024).  winv (with
// oz_ring): the transposed inverses of the diagonal factor tiles are kept
// there, tile k at winv + k nb^2 (ld = its row count), all mt of them.
void build_cholesky_region(dg_region *r, char uplo, int n, int nb, double *const *tiles,
                           void *oz_ring = nullptr, double *winv = nullptr);
// Upload tasks for every tile from a row-major source (element (r, c) at
// host[r*ldh + c]), ranked like the factorization's first use of the tile;
// added before build_cholesky_region, its tasks then wait only for the
// tiles they touch.
// Workspace of the tiled LU of an m x n matrix in nb x nb tiles (byte
// offsets from its base): the status and info words, the leaf launches'
// scratch, every panel's pivots (panel rows) and interchange row list, two
// panel buffers, the panel's emulated-update scratch and (emulated engine)
// the slice slots of the trailing updates.
struct LuLayout {
  size_t status = 0, info = 4, leaf = 256, lpiv = 0, lists = 0, panel = 0, panel_bytes = 0,
         ozp = 0, ozp_bytes = 0, ring = 0, winv = 0, winv_bytes = 0, ipiv = 0, total = 0;
  int list_cap = 0;        // entries of one step's destination (and source) list
  size_t list_stride = 0;  // ints per step
};
LuLayout lu_layout(int m, int n, int nb, bool pivot, bool emulated);
// The datadeps region of lu!(A, RowMaximum()) (pivot) or lu!(A, NoPivot())
// (src/array/lu.jl:5-54, 306-410) over the mt x nt tile grid; ws holds
// lu_layout(m, n, nb, pivot, emulated).total bytes; ipiv (device, min(m, n)
// int64) receives the global 1-based pivots (the entry point passes the
// workspace's copy, so that the graph does not depend on the caller's
// buffer).
void build_lu_region(dg_region *r, int m, int n, int nb, double *const *tiles, bool pivot,
                     void *ws, long long *ipiv, bool emulated);
// ldiv!(F::LU, B) (linalg.jl:264-308): B's rows permuted by ipiv, then the
// unit-lower and the upper block solves.  ws: lu_solve_bytes(n, nb, nrhs,
// emulated) bytes (the permutation, the permuted block columns, the slice
// slots of the emulated updates).
size_t lu_solve_bytes(int n, int nb, int nrhs, bool emulated);
// Offset of the pivots' copy in that workspace.
size_t lu_solve_ipiv_offset(int n, int nb, int nrhs, bool emulated);
void build_lu_solve_region(dg_region *r, int n, int nb, double *const *tiles,
                           const long long *ipiv, int nrhs, double *const *btiles, void *ws,
                           bool emulated);

// A copy of `ptrs` owned by the region (alive until it is destroyed), for
// tasks that address a list of tiles.
double *const *region_table(dg_region *r, const std::vector<double *> &ptrs);

void build_upload_tasks(dg_region *r, char uplo, int n, int nb, double *const *tiles,
                        const double *host, long long ldh);
// The datadeps regions of gemm_dagger! and syrk_dagger! + copytri!
// (src/array/mul.jl:133-425) over square nb x nb tile grids (column-major
// grids, ragged last row/column).  oz_ring (mul_ring_bytes_for bytes) selects
// the emulated FP64 products: each step of the contraction cuts its tiles'
// vectors into slices once, into a ring of kOzRingDepth steps.
size_t mul_ring_bytes_for(int m, int n, int nb);
void build_gemm_region(dg_region *r, char ta, char tb, int m, int n, int k, int nb, double alpha,
                       double *const *A, double *const *B, double beta, double *const *C,
                       void *oz_ring);
void build_syrk_region(dg_region *r, char trans, int n, int k, int nb, double alpha,
                       double *const *A, double beta, double *const *C, void *oz_ring);
// One block-triangular solve pass; oz_ring (oz_solve_ring_bytes_for bytes)
// selects emulated updates, step0 numbers its steps within the ring; winv
// (with oz_ring, the factorization's inverses) turns each diagonal block
// solve into one emulated product.
size_t oz_solve_ring_bytes_for(int n, int nb, int nrhs, bool inv = false);
void build_solve_pass(dg_region *r, char uplo, char trans, int n, int nb, double *const *tiles,
                      int nrhs, double *const *btiles, void *oz_ring = nullptr, int step0 = 0,
                      const double *winv = nullptr, char diag = 'N');

}  // namespace dg
