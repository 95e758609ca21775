// Out-of-core operator: FP32 A in host RAM (pinned) or in a raw file, streamed
// to the GPU tile by tile for every product.
//
// Replaces MPDOKOOCSolver (mpdok_ooc.py:51-383): build (:75-154) assembles
// FP32 row tiles on the GPU and stores them row-major without a header
// (RAM: np.empty((N,N),f32) at :117; SSD: tile.tofile at :142); the inner
// GMRES multiplies with a tiled SGEMV that copies every tile host -> device
// (:158-195, synchronous and pageable in the reference); the outer FP64
// residual is recomputed matrix-free from the coordinates (:205-227).
//
// Here the tiles sit in pinned memory and a side stream copies tile t+1 (and
// t+2) while the compute stream multiplies tile t (ring of OOC_NBUF device
// buffers, events in both directions), so the product runs at the host-link
// rate.  The file store reads each tile into a pinned staging slot with
// pread() before the device copy.  The outer residual uses the FP64 matrix-free
// kernel (matfree.cu).
#include "gemv.cuh"
#include "krylov.cuh"
#include "matfree.cuh"

#include <cerrno>
#include <cstdio>
#include <cstring>
#include <fcntl.h>
#include <string>
#include <thread>
#include <unistd.h>
#include <vector>

namespace mpdok {

constexpr int OOC_NBUF = 3;

struct OocHandle {
  long long n = 0;
  int tile_rows = 4096;
  int ntiles = 0;
  int store = 0;            // 0 = pinned host RAM, 1 = raw file
  std::string path;
  int fd = -1;
  float* host = nullptr;    // RAM store: N x N row-major FP32 (pinned)
  float* stage[OOC_NBUF] = {nullptr, nullptr, nullptr};  // file store: pinned staging
  float* dtile[OOC_NBUF] = {nullptr, nullptr, nullptr};
  cudaStream_t copy = nullptr;
  cudaEvent_t copied[OOC_NBUF] = {};
  cudaEvent_t consumed[OOC_NBUF] = {};
  void* gw = nullptr;       // GEMV workspace for one tile
  size_t gbytes = 0;
  double bytes_moved = 0.0;
};

static size_t tile_elems(const OocHandle* h) { return (size_t)h->tile_rows * (size_t)h->n; }

// pread of [off, off + bytes) into dst, retried until complete.
static int pread_all(int fd, char* dst, size_t bytes, off_t off) {
  size_t done = 0;
  while (done < bytes) {
    const ssize_t got = pread(fd, dst + done, bytes - done, off + (off_t)done);
    if (got < 0 && errno == EINTR) continue;
    if (got <= 0) return got == 0 ? -1 : errno;
    done += (size_t)got;
  }
  return 0;
}

// One tile from the file store into pinned staging.  A single reader thread
// tops out near 15 GB/s from the page cache, so the tile is split into 1 MiB
// aligned chunks read by up to OOC_READERS threads.
constexpr int OOC_READERS = 8;

static int ooc_read_tile(OocHandle* h, int t, float* dst) {
  const long long r0 = (long long)t * h->tile_rows;
  const long long rows = std::min<long long>(h->tile_rows, h->n - r0);
  const size_t bytes = (size_t)rows * h->n * sizeof(float);
  const off_t off = (off_t)r0 * h->n * (off_t)sizeof(float);
  const size_t chunk = 1u << 20;
  const int nthr = (int)std::min<size_t>(OOC_READERS, (bytes + chunk - 1) / chunk);
  std::vector<int> err(nthr, 0);
  auto worker = [&](int w) {
    // contiguous share of whole chunks per thread
    const size_t nch = (bytes + chunk - 1) / chunk;
    const size_t c0 = nch * w / nthr, c1 = nch * (w + 1) / nthr;
    const size_t b0 = c0 * chunk, b1 = std::min(bytes, c1 * chunk);
    if (b1 > b0) err[w] = pread_all(h->fd, (char*)dst + b0, b1 - b0, off + (off_t)b0);
  };
  std::vector<std::thread> pool;
  for (int w = 1; w < nthr; ++w) pool.emplace_back(worker, w);
  worker(0);
  for (auto& th : pool) th.join();
  for (int w = 0; w < nthr; ++w) {
    if (err[w]) {
      set_error("reading tile %d of %s failed (%s)", t, h->path.c_str(),
                err[w] < 0 ? "short file" : strerror(err[w]));
      return MPDOK_ERR_IO;
    }
  }
  return MPDOK_OK;
}

// y = A x with A streamed from the store.  x, y FP32 device vectors.
int ooc_matvec(OocHandle* h, const float* x, float* y, cudaStream_t s) {
  const long long n = h->n;
  MPDOK_CUDA_TRY(cudaEventRecord(h->consumed[0], s));  // the copy stream starts after prior work on s
  MPDOK_CUDA_TRY(cudaStreamWaitEvent(h->copy, h->consumed[0], 0));
  for (int b = 0; b < OOC_NBUF; ++b) MPDOK_CUDA_TRY(cudaEventRecord(h->consumed[b], s));
  auto issue = [&](int t) -> int {
    const int b = t % OOC_NBUF;
    const long long r0 = (long long)t * h->tile_rows;
    const long long rows = std::min<long long>(h->tile_rows, n - r0);
    const size_t bytes = (size_t)rows * n * sizeof(float);
    MPDOK_CUDA_TRY(cudaStreamWaitEvent(h->copy, h->consumed[b], 0));
    const float* src;
    if (h->store == 0) {
      src = h->host + (size_t)r0 * n;
    } else {
      // the staging slot b is free once the copy that last used it finished
      MPDOK_CUDA_TRY(cudaEventSynchronize(h->copied[b]));
      MPDOK_TRY(ooc_read_tile(h, t, h->stage[b]));
      src = h->stage[b];
    }
    const int slot = prof_start(MPDOK_PROF_OOC_COPY, h->copy);
    MPDOK_CUDA_TRY(cudaMemcpyAsync(h->dtile[b], src, bytes, cudaMemcpyHostToDevice, h->copy));
    prof_stop(slot, h->copy, (double)bytes);
    MPDOK_CUDA_TRY(cudaEventRecord(h->copied[b], h->copy));
    h->bytes_moved += (double)bytes;
    return MPDOK_OK;
  };
  const int lookahead = std::min(OOC_NBUF - 1, h->ntiles);
  for (int t = 0; t < lookahead; ++t) MPDOK_TRY(issue(t));
  for (int t = 0; t < h->ntiles; ++t) {
    if (t + lookahead < h->ntiles) MPDOK_TRY(issue(t + lookahead));
    const int b = t % OOC_NBUF;
    const long long r0 = (long long)t * h->tile_rows;
    const long long rows = std::min<long long>(h->tile_rows, n - r0);
    MPDOK_CUDA_TRY(cudaStreamWaitEvent(s, h->copied[b], 0));
    // tile (rows x n, row-major) = column-major (n x rows): y[r0:r0+rows] = tile^T-view . x
    MPDOK_TRY(gemv_launch(MPDOK_F32, true, h->dtile[b], n, n, rows, x, n, 1, y + r0, rows, 1.0, 0.0, nullptr, 0,
                          nullptr, h->gw, h->gbytes, s, false, nullptr));
    MPDOK_CUDA_TRY(cudaEventRecord(h->consumed[b], s));
  }
  return MPDOK_OK;
}

static int ooc_apply32(const void* ctx, const float* x, float* y, int nrhs, long long ld, cudaStream_t s,
                       const int* skip) {
  OocHandle* h = (OocHandle*)ctx;
  if (skip) {
    // Streaming costs a full pass over the host link: ask the device first.
    int hv = 0;
    MPDOK_CUDA_TRY(cudaMemcpyAsync(&hv, skip, sizeof(int), cudaMemcpyDeviceToHost, s));
    MPDOK_CUDA_TRY(cudaStreamSynchronize(s));
    if (hv) return MPDOK_OK;
  }
  for (int c = 0; c < nrhs; ++c) MPDOK_TRY(ooc_matvec(h, x + (long long)c * ld, y + (long long)c * ld, s));
  return MPDOK_OK;
}

}  // namespace mpdok

using namespace mpdok;

extern "C" int mpdok_ooc_create(long long n, int tile_rows, int store, const char* path, void** handle) {
  MPDOK_ARG_CHECK(handle != nullptr, "null handle pointer");
  *handle = nullptr;
  MPDOK_ARG_CHECK(n > 0 && tile_rows > 0, "n and tile_rows must be positive");
  MPDOK_ARG_CHECK(store == 0 || (store == 1 && path && *path), "store 1 (file) needs a path");
  OocHandle* h = new OocHandle();
  h->n = n;
  h->tile_rows = (int)std::min<long long>(tile_rows, n);
  h->ntiles = (int)((n + h->tile_rows - 1) / h->tile_rows);
  h->store = store;
  auto fail = [&](int st) {
    if (h->host) cudaFreeHost(h->host);
    for (int b = 0; b < OOC_NBUF; ++b) {
      if (h->stage[b]) cudaFreeHost(h->stage[b]);
      if (h->dtile[b]) cudaFree(h->dtile[b]);
      if (h->copied[b]) cudaEventDestroy(h->copied[b]);
      if (h->consumed[b]) cudaEventDestroy(h->consumed[b]);
    }
    if (h->copy) cudaStreamDestroy(h->copy);
    if (h->gw) cudaFree(h->gw);
    if (h->fd >= 0) close(h->fd);
    delete h;
    return st;
  };
  cudaError_t e;
  if (store == 0) {
    e = cudaHostAlloc((void**)&h->host, (size_t)n * (size_t)n * sizeof(float), cudaHostAllocDefault);
    if (e != cudaSuccess) {
      cuda_status(e, "cudaHostAlloc (OOC RAM store)");
      return fail(MPDOK_ERR_ALLOC);
    }
  } else {
    h->path = path;
    h->fd = open(path, O_RDWR | O_CREAT, 0644);
    if (h->fd < 0) {
      set_error("cannot open %s (%s)", path, strerror(errno));
      return fail(MPDOK_ERR_IO);
    }
    for (int b = 0; b < OOC_NBUF; ++b) {
      e = cudaHostAlloc((void**)&h->stage[b], tile_elems(h) * sizeof(float), cudaHostAllocDefault);
      if (e != cudaSuccess) { cuda_status(e, "cudaHostAlloc (OOC staging)"); return fail(MPDOK_ERR_ALLOC); }
    }
  }
  for (int b = 0; b < OOC_NBUF; ++b) {
    e = cudaMalloc((void**)&h->dtile[b], tile_elems(h) * sizeof(float));
    if (e != cudaSuccess) { cuda_status(e, "cudaMalloc (OOC tile)"); return fail(MPDOK_ERR_ALLOC); }
    if (cudaEventCreateWithFlags(&h->copied[b], cudaEventDisableTiming) != cudaSuccess ||
        cudaEventCreateWithFlags(&h->consumed[b], cudaEventDisableTiming) != cudaSuccess) {
      set_error("event creation failed");
      return fail(MPDOK_ERR_CUDA);
    }
  }
  if (cudaStreamCreateWithFlags(&h->copy, cudaStreamNonBlocking) != cudaSuccess) {
    set_error("copy stream creation failed");
    return fail(MPDOK_ERR_CUDA);
  }
  h->gbytes = gemv_workspace_bytes(MPDOK_F32, n, h->tile_rows, 1, true);
  e = cudaMalloc(&h->gw, h->gbytes);
  if (e != cudaSuccess) { cuda_status(e, "cudaMalloc (OOC GEMV workspace)"); return fail(MPDOK_ERR_ALLOC); }
  *handle = h;
  return MPDOK_OK;
}

extern "C" int mpdok_ooc_destroy(void* handle) {
  if (!handle) return MPDOK_OK;
  OocHandle* h = (OocHandle*)handle;
  cudaStreamSynchronize(h->copy);
  if (h->host) cudaFreeHost(h->host);
  for (int b = 0; b < OOC_NBUF; ++b) {
    if (h->stage[b]) cudaFreeHost(h->stage[b]);
    if (h->dtile[b]) cudaFree(h->dtile[b]);
    cudaEventDestroy(h->copied[b]);
    cudaEventDestroy(h->consumed[b]);
  }
  cudaStreamDestroy(h->copy);
  if (h->gw) cudaFree(h->gw);
  if (h->fd >= 0) close(h->fd);
  delete h;
  return MPDOK_OK;
}

// Assemble FP32 row tiles on the GPU (nugget on the global diagonal) and move
// them to the store, row-major without a header (mpdok_ooc.py:116-146).
extern "C" int mpdok_ooc_build(void* handle, const double* coords, int dim, int kernel, double gamma, double reg,
                               cudaStream_t s) {
  MPDOK_ARG_CHECK(handle && coords, "null pointer");
  MPDOK_ARG_CHECK(dim >= 1 && dim <= 3, "dim must be 1, 2 or 3");
  OocHandle* h = (OocHandle*)handle;
  const long long n = h->n;
  for (int t = 0; t < h->ntiles; ++t) {
    const long long r0 = (long long)t * h->tile_rows;
    const long long rows = std::min<long long>(h->tile_rows, n - r0);
    float* d = h->dtile[t % OOC_NBUF];
    MPDOK_TRY(rbf_tile_f32_from_f64(coords + r0 * dim, rows, coords, n, dim, kernel, gamma, reg, r0, d, n, s));
    const size_t bytes = (size_t)rows * n * sizeof(float);
    if (h->store == 0) {
      MPDOK_CUDA_TRY(cudaMemcpyAsync(h->host + (size_t)r0 * n, d, bytes, cudaMemcpyDeviceToHost, s));
    } else {
      float* st = h->stage[0];
      MPDOK_CUDA_TRY(cudaMemcpyAsync(st, d, bytes, cudaMemcpyDeviceToHost, s));
      MPDOK_CUDA_TRY(cudaStreamSynchronize(s));
      size_t done = 0;
      const off_t off = (off_t)r0 * n * (off_t)sizeof(float);
      while (done < bytes) {
        const ssize_t w = pwrite(h->fd, (const char*)st + done, bytes - done, off + (off_t)done);
        if (w <= 0) {
          set_error("writing tile %d to %s failed (%s)", t, h->path.c_str(), strerror(errno));
          return MPDOK_ERR_IO;
        }
        done += (size_t)w;
      }
    }
  }
  MPDOK_CUDA_TRY(cudaStreamSynchronize(s));
  if (h->store == 1 && fsync(h->fd) != 0) {
    set_error("fsync of %s failed (%s)", h->path.c_str(), strerror(errno));
    return MPDOK_ERR_IO;
  }
  return MPDOK_OK;
}

extern "C" int mpdok_ooc_matvec(void* handle, const float* x, float* y, cudaStream_t s) {
  MPDOK_ARG_CHECK(handle && x && y, "null pointer");
  return ooc_matvec((OocHandle*)handle, x, y, s);
}

// Host copy of rows [r0, r0 + rows) of the stored FP32 matrix (row-major).
extern "C" int mpdok_ooc_read_rows(void* handle, long long r0, long long rows, float* dst) {
  MPDOK_ARG_CHECK(handle && dst, "null pointer");
  OocHandle* h = (OocHandle*)handle;
  MPDOK_ARG_CHECK(r0 >= 0 && rows >= 0 && r0 + rows <= h->n, "row range outside the matrix");
  const size_t bytes = (size_t)rows * (size_t)h->n * sizeof(float);
  if (h->store == 0) {
    std::memcpy(dst, h->host + (size_t)r0 * h->n, bytes);
    return MPDOK_OK;
  }
  const int e = pread_all(h->fd, (char*)dst, bytes, (off_t)r0 * h->n * (off_t)sizeof(float));
  if (e) {
    set_error("reading %s failed (%s)", h->path.c_str(), e < 0 ? "short file" : strerror(e));
    return MPDOK_ERR_IO;
  }
  return MPDOK_OK;
}

extern "C" double mpdok_ooc_bytes_moved(void* handle) {
  return handle ? ((OocHandle*)handle)->bytes_moved : 0.0;
}

extern "C" size_t mpdok_ooc_workspace_size(long long n, int restart) {
  if (n < 0 || restart < 1) return 0;
  return krylov_layout(n, restart, nullptr).total + matfree_work_bytes(n, n, 1, MPDOK_F64) + 512;
}

// GMRES-IR of MPDOKOOCSolver.solve (mpdok_ooc.py:315-373): outer FP64 residual
// recomputed matrix-free from the coordinates, inner FP32 GMRES on the
// streamed operator (two Gram-Schmidt passes, FP64 Givens, |g|/beta < inner_tol).
extern "C" int mpdok_ooc_gmres_ir(void* handle, const double* coords, int dim, int kernel, double gamma, double reg,
                                  const double* b, double* x, double tol, int maxiter_outer, int restart,
                                  double inner_tol, void* work, size_t work_bytes, mpdok_solve_info* info,
                                  cudaStream_t s) {
  if (info) std::memset(info, 0, sizeof(*info));
  MPDOK_ARG_CHECK(handle && coords && b && x && work, "null pointer");
  MPDOK_ARG_CHECK(restart >= 1 && restart <= 1024, "restart must be in [1, 1024]");
  OocHandle* h = (OocHandle*)handle;
  const long long n = h->n;
  MPDOK_ARG_CHECK(work_bytes >= mpdok_ooc_workspace_size(n, restart), "OOC workspace too small");
  KWs ws = krylov_layout(n, restart, work);
  MPDOK_TRY(ws_prepare(ws, work_bytes, s));
  MfCtx c;
  c.op.rows = coords;
  c.op.cols = coords;
  c.op.nrows = n;
  c.op.ncols = n;
  c.op.dim = dim;
  c.op.kernel = kernel;
  c.op.gamma = gamma;
  c.op.reg = reg;
  c.w64 = (char*)work + align_up(ws.total, 256);
  c.w64_bytes = matfree_work_bytes(n, n, 1, MPDOK_F64);
  Operator32 A;
  A.apply = ooc_apply32;
  A.ctx = h;
  return gmres_ir_core(ws, A, mf_res64(&c), b, x, tol, maxiter_outer, restart, inner_tol, nullptr, info, s);
}
