// Device-resident Krylov solvers (GMRES-IR, restarted GMRES, CG) for sm_103a.
//
// The reference runs these loops in Python with a host round trip per
// iteration (float(cp.dot(...)) at dense_krylov.py:192,195; cp.asnumpy(h) at
// dense_krylov.py:292 and mpdok_ooc.py:265,272; float(cp.linalg.norm(w)) at
// dense_krylov.py:295 and mpdok_ooc.py:275).  Here the Arnoldi / CG state
// (Hessenberg matrix, Givens rotations, step lengths) lives on the device in
// FP64, every kernel of a cycle is predicated on a device `done` flag, and the
// host reads one small struct per outer step (or per restart / CG check).
//
// Reductions are two-level and ordered (per-block parts summed by the last
// block in block-index order), so every solve is bitwise reproducible.
#include "krylov.cuh"

#include <cmath>
#include <cstring>
#include <limits>
#include <vector>

namespace mpdok {

constexpr int KT = 256;
constexpr int KMAX_RESTART = 1024;

__device__ __forceinline__ bool last_block_arrive(unsigned* ticket) {
  __shared__ bool s_last;
  __threadfence();
  __syncthreads();
  if (threadIdx.x == 0) {
    unsigned t = atomicAdd(ticket, 1u);
    s_last = (t == gridDim.x * gridDim.y - 1);
  }
  __syncthreads();
  if (s_last) __threadfence();
  return s_last;
}

struct ArnState {
  double* H;   // (m+1) x m, column-major, ldh = m+1
  long long ldh;
  double* cs;
  double* sn;
  double* g;
  double* y;
};

// Per-block dot products of V[:, 0..kp1) (rows of this chunk) with sw.
__device__ __forceinline__ void block_dots(const float* Vc, long long ldv, int kp1, const float* sw, int len,
                                           double* part_out) {
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nw = blockDim.x >> 5;
  for (int j = warp; j < kp1; j += nw) {
    const float* v = Vc + (long long)j * ldv;
    double acc = 0.0;
    for (int i = lane; i < len; i += 32) acc = fma((double)v[i], (double)sw[i], acc);
    acc = warp_sum(acc);
    if (lane == 0) part_out[j] = acc;
  }
}

// Ordered column sums of parts[b * kp1 + j] over blocks b, by the last block.
__device__ __forceinline__ void finish_dots(const double* parts, int nb, int kp1, double* out, double* accum) {
  for (int j = threadIdx.x; j < kp1; j += blockDim.x) {
    double s = 0.0;
    for (int b = 0; b < nb; ++b) s += __ldcg(parts + (long long)b * kp1 + j);
    out[j] = s;
    if (accum) accum[j] += s;
  }
}

// h = V[:, :kp1]^T w  (first Gram-Schmidt pass), stored into `out`.
__global__ void __launch_bounds__(KT)
k_dots(const float* __restrict__ V, long long ldv, int kp1, const float* __restrict__ w, long long n, long long ch,
       double* parts, unsigned* ticket, double* out, const KScal* sc) {
  extern __shared__ float sw[];
  if (sc->done) return;
  const long long r0 = (long long)blockIdx.x * ch;
  const int len = (int)min(ch, n - r0);
  for (int t = threadIdx.x; t < len; t += blockDim.x) sw[t] = w[r0 + t];
  __syncthreads();
  block_dots(V + r0, ldv, kp1, sw, len, parts + (long long)blockIdx.x * kp1);
  if (last_block_arrive(ticket)) {
    finish_dots(parts, gridDim.x, kp1, out, nullptr);
    if (threadIdx.x == 0) *ticket = 0u;
  }
}

// Arnoldi step finish (one thread): H(k+1,k), previous rotations, new Givens
// rotation, residual estimate g, stop flags.  mpdok_ooc.py:275-301.
__device__ void arnoldi_finish(KScal* sc, const ArnState& st, int k, double nrm2, double tol_rel) {
  double* H = st.H;
  const long long ldh = st.ldh;
  const double nrm = sqrt(nrm2);
  H[(k + 1) + k * ldh] = nrm;
  const bool bd = !(nrm > 1e-12);
  for (int j = 0; j < k; ++j) {
    const double hj = H[j + k * ldh], hj1 = H[(j + 1) + k * ldh];
    const double tmp = st.cs[j] * hj + st.sn[j] * hj1;
    H[(j + 1) + k * ldh] = -st.sn[j] * hj + st.cs[j] * hj1;
    H[j + k * ldh] = tmp;
  }
  const double a = H[k + k * ldh], b = H[(k + 1) + k * ldh];
  const double rho = hypot(a, b);
  double c = 1.0, s = 0.0;
  if (rho != 0.0) { c = a / rho; s = b / rho; }
  st.cs[k] = c;
  st.sn[k] = s;
  H[k + k * ldh] = (rho != 0.0) ? rho : a;
  H[(k + 1) + k * ldh] = 0.0;
  st.g[k + 1] = -s * st.g[k];
  st.g[k] = c * st.g[k];
  sc->m_used = k + 1;
  sc->aux = nrm;
  if (!isfinite(nrm) || !isfinite(st.g[k + 1])) {
    sc->nonfinite = 1;
    sc->done = 1;
  } else if (bd) {
    sc->breakdown = 1;
    sc->done = 1;
  } else if (tol_rel > 0.0 && fabs(st.g[k + 1]) / sc->beta < tol_rel) {
    sc->done = 1;
  }
}

// w -= V[:, :kp1] h, then either the second-pass dots (MODE 0) or ||w||^2 and
// the step finish (MODE 1).
template <int MODE>
__global__ void __launch_bounds__(KT)
k_apply(const float* __restrict__ V, long long ldv, int kp1, float* __restrict__ w, long long n, long long ch,
        const double* h, double* parts, unsigned* ticket, double* h2out, double* Hcol, KScal* sc, ArnState st,
        int k, double tol_rel) {
  extern __shared__ float smem[];
  float* sh = smem;             // kp1 floats
  float* sw = smem + KMAX_RESTART + 1;  // ch floats
  __shared__ double red[32];
  if (sc->done) return;
  for (int j = threadIdx.x; j < kp1; j += blockDim.x) sh[j] = (float)h[j];
  __syncthreads();
  const long long r0 = (long long)blockIdx.x * ch;
  const int len = (int)min(ch, n - r0);
  double sq = 0.0;
  for (int t = threadIdx.x; t < len; t += blockDim.x) {
    const float* v = V + r0 + t;
    float acc = 0.f;
    for (int j = 0; j < kp1; ++j) acc = fmaf(v[(long long)j * ldv], sh[j], acc);
    const float nw = w[r0 + t] - acc;
    w[r0 + t] = nw;
    if (MODE == 0) sw[t] = nw;
    else sq = fma((double)nw, (double)nw, sq);
  }
  if (MODE == 0) {
    __syncthreads();
    block_dots(V + r0, ldv, kp1, sw, len, parts + (long long)blockIdx.x * kp1);
    if (last_block_arrive(ticket)) {
      finish_dots(parts, gridDim.x, kp1, h2out, Hcol);
      if (threadIdx.x == 0) *ticket = 0u;
    }
  } else {
    const double bsum = block_sum(sq, red);
    if (threadIdx.x == 0) parts[blockIdx.x] = bsum;
    if (last_block_arrive(ticket)) {
      if (threadIdx.x < 32) {
        double s = 0.0;
        for (unsigned b = threadIdx.x; b < gridDim.x; b += 32) s += __ldcg(parts + b);
        s = warp_sum(s);
        if (threadIdx.x == 0) {
          sc->nrm2 = s;
          arnoldi_finish(sc, st, k, s, tol_rel);
          *ticket = 0u;
        }
      }
    }
  }
}

// V[:, k+1] = w * (1 / ||w||)  (mpdok_ooc.py:279).
__global__ void k_normalize(const float* __restrict__ w, float* __restrict__ vnext, long long n, const KScal* sc) {
  if (sc->done) return;
  const float inv = (float)(1.0 / sc->aux);
  for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x)
    vnext[i] = w[i] * inv;
}

// dst = (float) src with ||dst||^2, then the cycle state: beta, g[0], flags.
template <typename S>
__global__ void __launch_bounds__(KT)
k_cast_start(const S* __restrict__ src, float* __restrict__ dst, long long n, double* parts, unsigned* ticket,
             KScal* sc, double* g) {
  __shared__ double red[32];
  double sq = 0.0;
  for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x) {
    const float v = (float)src[i];
    dst[i] = v;
    sq = fma((double)v, (double)v, sq);
  }
  const double bsum = block_sum(sq, red);
  if (threadIdx.x == 0) parts[blockIdx.x] = bsum;
  if (last_block_arrive(ticket)) {
    if (threadIdx.x < 32) {
      double s = 0.0;
      for (unsigned b = threadIdx.x; b < gridDim.x; b += 32) s += __ldcg(parts + b);
      s = warp_sum(s);
      if (threadIdx.x == 0) {
        const double beta = sqrt(s);
        sc->nrm2 = s;
        sc->beta = beta;
        g[0] = beta;
        sc->m_used = 0;
        sc->breakdown = 0;
        sc->nonfinite = isfinite(beta) ? 0 : 1;
        sc->done = (beta < 1e-30 || !isfinite(beta)) ? 1 : 0;
        *ticket = 0u;
      }
    }
  }
}

__global__ void k_scale_v0(float* __restrict__ v, long long n, const KScal* sc) {
  if (sc->done) return;
  const float inv = (float)(1.0 / sc->beta);
  for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x)
    v[i] *= inv;
}

// y = H(0:m,0:m)^{-1} g(0:m) by back substitution (mpdok_ooc.py:303-307).
__global__ void k_backsub(const KScal* sc, ArnState st) {
  if (threadIdx.x != 0) return;
  const int m = sc->m_used;
  const long long ldh = st.ldh;
  for (int j = m - 1; j >= 0; --j) {
    double s = st.g[j];
    for (int l = j + 1; l < m; ++l) s -= st.H[j + l * ldh] * st.y[l];
    const double d = st.H[j + j * ldh];
    st.y[j] = (d != 0.0) ? s / d : 0.0;
  }
}

// x += V[:, :m] y with the product in FP32 (mpdok_ooc.py:310, :365).
template <typename TX>
__global__ void k_update(const float* __restrict__ V, long long ldv, const double* __restrict__ y, const KScal* sc,
                         long long n, TX* __restrict__ x, float* __restrict__ tout) {
  __shared__ float sy[KMAX_RESTART];
  const int m = sc->m_used;
  if (m == 0) return;
  for (int j = threadIdx.x; j < m; j += blockDim.x) sy[j] = (float)y[j];
  __syncthreads();
  for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x) {
    float acc = 0.f;
    for (int j = 0; j < m; ++j) acc = fmaf(V[i + (long long)j * ldv], sy[j], acc);
    if (tout) tout[i] = acc;
    else x[i] = (TX)(x[i] + (TX)acc);
  }
}

template <typename TX>
__global__ void k_axpy_f32(const float* __restrict__ t, long long n, TX* __restrict__ x, const KScal* sc) {
  if (sc->m_used == 0) return;
  for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x)
    x[i] = (TX)(x[i] + (TX)t[i]);
}

template <typename T>
__global__ void __launch_bounds__(KT)
k_norm2(const T* __restrict__ x, long long n, double* parts, unsigned* ticket, double* out) {
  __shared__ double red[32];
  double sq = 0.0;
  for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x) {
    const double v = (double)x[i];
    sq = fma(v, v, sq);
  }
  ordered_grid_sum(block_sum(sq, red), parts, ticket, out);
}

// nrm2[c] = ||r[:, c]||^2, one block per column (fixed reduction order).
__global__ void __launch_bounds__(KT) k_colnorms(const double* __restrict__ r, long long n, long long ld,
                                                 double* nrm2) {
  __shared__ double red[32];
  const double* col = r + (long long)blockIdx.x * ld;
  double s = 0.0;
  for (long long i = threadIdx.x; i < n; i += blockDim.x) s = fma(col[i], col[i], s);
  s = block_sum(s, red);
  if (threadIdx.x == 0) nrm2[blockIdx.x] = s;
}

// w = b - w (the FP32 residual of a GMRES restart)
__global__ void k_sub_from(const float* __restrict__ b, float* __restrict__ w, long long n) {
  for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x)
    w[i] = b[i] - w[i];
}

__global__ void k_axpy_f64(const double* __restrict__ e, double* __restrict__ x, long long n) {
  for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x)
    x[i] += e[i];
}

// ----------------------------------------------------------------- CG kernels
// alpha = rs / (p . q)  (dense_krylov.py:192)
__global__ void __launch_bounds__(KT)
k_cg_pap(const float* __restrict__ p, const float* __restrict__ q, long long n, double* parts, unsigned* ticket,
         KScal* sc) {
  __shared__ double red[32];
  if (sc->done) return;
  double acc = 0.0;
  for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x)
    acc = fma((double)p[i], (double)q[i], acc);
  const double bsum = block_sum(acc, red);
  if (threadIdx.x == 0) parts[blockIdx.x] = bsum;
  if (last_block_arrive(ticket)) {
    if (threadIdx.x < 32) {
      double s = 0.0;
      for (unsigned b = threadIdx.x; b < gridDim.x; b += 32) s += __ldcg(parts + b);
      s = warp_sum(s);
      if (threadIdx.x == 0) {
        // The reference takes the FP32 dot (cp.dot of FP32 vectors).
        const double pap = (double)(float)s;
        if (pap == 0.0 || !isfinite(pap)) {
          sc->alpha = 0.0;
          sc->done = 1;
          sc->breakdown = 1;
        } else {
          sc->alpha = sc->rs / pap;
        }
        *ticket = 0u;
      }
    }
  }
}

// x += alpha p; r -= alpha q; rs_new = r.r; beta = rs_new / rs  (dense_krylov.py:193-198)
__global__ void __launch_bounds__(KT)
k_cg_xr(float* __restrict__ x, float* __restrict__ r, const float* __restrict__ p, const float* __restrict__ q,
        long long n, double* parts, unsigned* ticket, KScal* sc) {
  __shared__ double red[32];
  if (sc->done) return;
  const float a = (float)sc->alpha;
  double acc = 0.0;
  for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x) {
    x[i] = x[i] + a * p[i];
    const float rn = r[i] - a * q[i];
    r[i] = rn;
    acc = fma((double)rn, (double)rn, acc);
  }
  const double bsum = block_sum(acc, red);
  if (threadIdx.x == 0) parts[blockIdx.x] = bsum;
  if (last_block_arrive(ticket)) {
    if (threadIdx.x < 32) {
      double s = 0.0;
      for (unsigned b = threadIdx.x; b < gridDim.x; b += 32) s += __ldcg(parts + b);
      s = warp_sum(s);
      if (threadIdx.x == 0) {
        const double rs_new = (double)(float)s;
        sc->betacg = (sc->rs != 0.0) ? rs_new / sc->rs : 0.0;
        sc->rs = rs_new;
        if (!isfinite(rs_new)) { sc->nonfinite = 1; sc->done = 1; }
        *ticket = 0u;
      }
    }
  }
}

__global__ void k_cg_p(float* __restrict__ p, const float* __restrict__ r, long long n, const KScal* sc) {
  if (sc->done) return;
  const float b = (float)sc->betacg;
  for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x)
    p[i] = r[i] + b * p[i];
}

__global__ void k_set_rs(KScal* sc) {
  if (threadIdx.x == 0) {
    sc->rs = (double)(float)sc->nrm2;
    sc->done = 0;
    sc->breakdown = 0;
    sc->nonfinite = 0;
  }
}

// --------------------------------------------------- multi-RHS CG (CG-IR inner)
// Columns advance in lockstep so that every operator application reads A once
// for all of them; each column has its own step lengths and stops on its own
// relative tolerance (a stopped column keeps alpha = 0).
struct MColState {
  double rs, alpha, beta, r0, rz;
  int done;
  int pad;
};

struct MCGGlobal {
  int done;        // every column reached the inner tolerance
  int iters;
};

// One block per (row chunk, column); per-column ordered reduction by the last block.
__device__ __forceinline__ bool last_block_all(unsigned* ticket) {
  __shared__ bool s_last;
  __threadfence();
  __syncthreads();
  if (threadIdx.x == 0) {
    unsigned t = atomicAdd(ticket, 1u);
    s_last = (t == gridDim.x * gridDim.y - 1);
  }
  __syncthreads();
  if (s_last) __threadfence();
  return s_last;
}

__global__ void __launch_bounds__(KT)
k_mcg_init(const double* __restrict__ R64, long long ld, long long n, float* E, float* r, float* p, double* parts,
           unsigned* ticket, MColState* cols, MCGGlobal* g) {
  __shared__ double red[32];
  const int c = blockIdx.y;
  double acc = 0.0;
  for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x) {
    const float v = (float)R64[i + c * ld];
    E[i + c * ld] = 0.f;
    r[i + c * ld] = v;
    p[i + c * ld] = v;
    acc = fma((double)v, (double)v, acc);
  }
  const double b = block_sum(acc, red);
  if (threadIdx.x == 0) parts[(long long)c * gridDim.x + blockIdx.x] = b;
  if (last_block_all(ticket)) {
    if (threadIdx.x < gridDim.y) {
      const int cc = threadIdx.x;
      double t = 0.0;
      for (unsigned k = 0; k < gridDim.x; ++k) t += __ldcg(parts + (long long)cc * gridDim.x + k);
      cols[cc].rs = t;
      cols[cc].rz = t;
      cols[cc].r0 = sqrt(t);
      cols[cc].done = (t == 0.0) ? 1 : 0;
      cols[cc].alpha = cols[cc].beta = 0.0;
    }
    __syncthreads();
    if (threadIdx.x == 0) {
      int all = 1;
      for (unsigned cc = 0; cc < gridDim.y; ++cc) all &= cols[cc].done;
      g->done = all;
      g->iters = 0;
      *ticket = 0u;
    }
  }
}

__global__ void __launch_bounds__(KT)
k_mcg_pap(const float* __restrict__ p, const float* __restrict__ q, long long ld, long long n, double* parts,
          unsigned* ticket, MColState* cols, const MCGGlobal* g) {
  __shared__ double red[32];
  if (g->done) return;
  const int c = blockIdx.y;
  double acc = 0.0;
  for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x)
    acc = fma((double)p[i + c * ld], (double)q[i + c * ld], acc);
  const double b = block_sum(acc, red);
  if (threadIdx.x == 0) parts[(long long)c * gridDim.x + blockIdx.x] = b;
  if (last_block_all(ticket)) {
    if (threadIdx.x < gridDim.y) {
      const int cc = threadIdx.x;
      double t = 0.0;
      for (unsigned k = 0; k < gridDim.x; ++k) t += __ldcg(parts + (long long)cc * gridDim.x + k);
      if (cols[cc].done || !(t > 0.0) || !isfinite(t)) {
        cols[cc].alpha = 0.0;
        if (!cols[cc].done && !(t > 0.0)) cols[cc].done = 1;
      } else {
        cols[cc].alpha = cols[cc].rz / t;
      }
    }
    if (threadIdx.x == 0) *ticket = 0u;
  }
}

__global__ void __launch_bounds__(KT)
k_mcg_xr(float* E, float* r, const float* __restrict__ p, const float* __restrict__ q, long long ld, long long n,
         double* parts, unsigned* ticket, MColState* cols, MCGGlobal* g, double inner_tol, int precond) {
  __shared__ double red[32];
  if (g->done) return;
  const int c = blockIdx.y;
  const float a = (float)cols[c].alpha;
  double acc = 0.0;
  for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x) {
    const long long k = i + c * ld;
    E[k] = fmaf(a, p[k], E[k]);
    const float rn = fmaf(-a, q[k], r[k]);
    r[k] = rn;
    acc = fma((double)rn, (double)rn, acc);
  }
  const double b = block_sum(acc, red);
  if (threadIdx.x == 0) parts[(long long)c * gridDim.x + blockIdx.x] = b;
  if (last_block_all(ticket)) {
    if (threadIdx.x < gridDim.y) {
      const int cc = threadIdx.x;
      double t = 0.0;
      for (unsigned k = 0; k < gridDim.x; ++k) t += __ldcg(parts + (long long)cc * gridDim.x + k);
      if (!cols[cc].done) {
        if (!precond) {
          cols[cc].beta = (cols[cc].rz > 0.0) ? t / cols[cc].rz : 0.0;
          cols[cc].rz = t;
        }
        cols[cc].rs = t;
        if (!(sqrt(t) > inner_tol * cols[cc].r0)) cols[cc].done = 1;
      } else {
        cols[cc].beta = 0.0;
      }
    }
    __syncthreads();
    if (threadIdx.x == 0) {
      int all = 1;
      for (unsigned cc = 0; cc < gridDim.y; ++cc) all &= cols[cc].done;
      g->done = all;
      g->iters += 1;
      *ticket = 0u;
    }
  }
}

// rz_new = r . z per column; initial (init != 0): rz = rz_new; else beta = rz_new / rz, rz = rz_new.
__global__ void __launch_bounds__(KT)
k_mcg_rz(const float* __restrict__ r, const float* __restrict__ z, long long ld, long long n, double* parts,
         unsigned* ticket, MColState* cols, const MCGGlobal* g, int init) {
  __shared__ double red[32];
  if (!init && g->done) return;
  const int c = blockIdx.y;
  double acc = 0.0;
  for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x)
    acc = fma((double)r[i + c * ld], (double)z[i + c * ld], acc);
  const double b = block_sum(acc, red);
  if (threadIdx.x == 0) parts[(long long)c * gridDim.x + blockIdx.x] = b;
  if (last_block_all(ticket)) {
    if (threadIdx.x < gridDim.y) {
      const int cc = threadIdx.x;
      double t = 0.0;
      for (unsigned k = 0; k < gridDim.x; ++k) t += __ldcg(parts + (long long)cc * gridDim.x + k);
      if (init) {
        cols[cc].rz = t;
      } else if (!cols[cc].done) {
        cols[cc].beta = (cols[cc].rz != 0.0) ? t / cols[cc].rz : 0.0;
        cols[cc].rz = t;
      }
    }
    if (threadIdx.x == 0) *ticket = 0u;
  }
}

__global__ void k_mcg_p(float* p, const float* __restrict__ r, long long ld, long long n, const MColState* cols,
                        const MCGGlobal* g) {
  if (g->done) return;
  const int c = blockIdx.y;
  if (cols[c].done) return;
  const float bt = (float)cols[c].beta;
  for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x)
    p[i + c * ld] = fmaf(bt, p[i + c * ld], r[i + c * ld]);
}

__global__ void k_add_cols(const float* __restrict__ E, long long lde, double* X, long long ldx, long long n) {
  const int c = blockIdx.y;
  for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x)
    X[i + c * ldx] += (double)E[i + c * lde];
}

__global__ void k_copy_cols(const double* __restrict__ src, long long lds, double* dst, long long ldd, long long n) {
  const int c = blockIdx.y;
  for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x)
    dst[i + c * ldd] = src[i + c * lds];
}

// ------------------------------------------------------------------ host side

int colnorms_f64(const double* r, long long n, int nrhs, long long ld, double* nrm2, cudaStream_t s) {
  launch(k_colnorms, nrhs, KT, 0, s, r, n, ld, nrm2);
  MPDOK_LAUNCH_CHECK("colnorms");
  return MPDOK_OK;
}

static unsigned vec_blocks(long long n) {
  long long b = (n + KT - 1) / KT;
  long long cap = (long long)num_sms() * 2;
  return (unsigned)std::max(1LL, std::min(b, cap));
}

KWs krylov_layout(long long n, int m, void* base) {
  KWs ws;
  ws.n = n;
  ws.m = m;
  ws.ldv = (long long)align_up((size_t)std::max(1LL, n), 64);
  const long long nsm = num_sms();
  long long ch = (n + 2 * nsm - 1) / (2 * nsm);
  ch = (long long)align_up((size_t)std::max(1LL, ch), 256);
  ch = std::min(std::max(ch, 256LL), 4096LL);
  ws.ch = ch;
  ws.nblk = (int)std::max(1LL, (n + ch - 1) / ch);
  size_t off = 0;
  auto take = [&](size_t bytes) { size_t o = off; off = align_up(off + bytes, 256); return o; };
  const size_t fv = (size_t)ws.ldv * sizeof(float);
  const size_t dv = (size_t)ws.ldv * sizeof(double);
  size_t oV = take(fv * (m + 1)), ow = take(fv), ox = take(fv), ob = take(fv), op = take(fv), oq = take(fv);
  size_t or64 = take(dv), ox64 = take(dv), oe64 = take(dv * 2);
  size_t oH = take(sizeof(double) * (size_t)(m + 1) * m), ocs = take(sizeof(double) * m),
         osn = take(sizeof(double) * m), og = take(sizeof(double) * (m + 1)), oy = take(sizeof(double) * m),
         oh2 = take(sizeof(double) * (m + 1));
  const size_t nparts = (size_t)std::max<long long>(ws.nblk, vec_blocks(n)) * (m + 1) + 64;
  size_t oparts = take(sizeof(double) * nparts);
  size_t otk = take(sizeof(unsigned) * 8);
  size_t osc = take(sizeof(KScal));
  ws.gbytes = std::max(gemv_workspace_bytes(MPDOK_F32, n, n, 1, false), gemv_workspace_bytes(MPDOK_F64, n, n, 1, false));
  size_t ogw = take(ws.gbytes);
  ws.total = off;
  if (base) {
    char* b = (char*)base;
    ws.V = (float*)(b + oV); ws.w = (float*)(b + ow); ws.x32 = (float*)(b + ox); ws.b32 = (float*)(b + ob);
    ws.p32 = (float*)(b + op); ws.q32 = (float*)(b + oq);
    ws.r64 = (double*)(b + or64); ws.x64t = (double*)(b + ox64); ws.e64 = (double*)(b + oe64);
    ws.H = (double*)(b + oH); ws.cs = (double*)(b + ocs); ws.sn = (double*)(b + osn); ws.g = (double*)(b + og);
    ws.y = (double*)(b + oy); ws.h2 = (double*)(b + oh2); ws.parts = (double*)(b + oparts);
    ws.tickets = (unsigned*)(b + otk); ws.sc = (KScal*)(b + osc); ws.gw = (void*)(b + ogw);
  }
  return ws;
}

static ArnState arn_state(const KWs& ws) {
  ArnState st;
  st.H = ws.H; st.ldh = ws.m + 1; st.cs = ws.cs; st.sn = ws.sn; st.g = ws.g; st.y = ws.y;
  return st;
}

static int stored_apply32(const void* ctx, const float* x, float* y, int nrhs, long long ld, cudaStream_t s,
                          const int* skip) {
  const StoredCtx* c = (const StoredCtx*)ctx;
  return gemv_launch(MPDOK_F32, false, c->A32, c->lda32, c->n, c->n, x, ld, nrhs, y, ld, 1.0, 0.0, nullptr, 0,
                     nullptr, c->gw, c->gbytes, s, false, skip);
}

static int stored_residual64(const void* ctx, const double* b, const double* x, double* r, double* nrm2, int nrhs,
                             long long ld, cudaStream_t s) {
  const StoredCtx* c = (const StoredCtx*)ctx;
  if (nrhs == 1)
    return gemv_launch(MPDOK_F64, false, c->A64, c->lda64, c->n, c->n, x, ld, 1, r, ld, -1.0, 1.0, b, ld, nrm2,
                       c->gw, c->gbytes, s, true, nullptr);
  MPDOK_TRY(gemv_launch(MPDOK_F64, false, c->A64, c->lda64, c->n, c->n, x, ld, nrhs, r, ld, -1.0, 1.0, b, ld,
                        nullptr, c->gw, c->gbytes, s, true, nullptr));
  return colnorms_f64(r, c->n, nrhs, ld, nrm2, s);
}

Operator32 stored_op32(const StoredCtx* c) {
  Operator32 o;
  o.apply = stored_apply32;
  o.ctx = c;
  return o;
}

Residual64 stored_res64(const StoredCtx* c) {
  Residual64 o;
  o.apply = stored_residual64;
  o.ctx = c;
  return o;
}

int read_scal(const KWs& ws, KScal* host, cudaStream_t s) {
  MPDOK_CUDA_TRY(cudaMemcpyAsync(host, ws.sc, sizeof(KScal), cudaMemcpyDeviceToHost, s));
  MPDOK_CUDA_TRY(cudaStreamSynchronize(s));
  return MPDOK_OK;
}

int norm2_f64(const KWs& ws, const double* x, long long n, double* out_dev, cudaStream_t s) {
  launch(k_norm2<double>, vec_blocks(n), KT, 0, s, x, n, ws.parts, ws.tickets + 4, out_dev);
  MPDOK_LAUNCH_CHECK("norm2");
  return MPDOK_OK;
}

int cycle_start_from_f64(const KWs& ws, const double* src64, cudaStream_t s) {
  launch(k_cast_start<double>, vec_blocks(ws.n), KT, 0, s, src64, ws.V, ws.n, ws.parts, ws.tickets + 5, ws.sc, ws.g);
  launch(k_scale_v0, vec_blocks(ws.n), KT, 0, s, ws.V, ws.n, ws.sc);
  MPDOK_LAUNCH_CHECK("cycle start");
  return MPDOK_OK;
}

static int cycle_start_from_f32(const KWs& ws, const float* src32, cudaStream_t s) {
  launch(k_cast_start<float>, vec_blocks(ws.n), KT, 0, s, src32, ws.V, ws.n, ws.parts, ws.tickets + 5, ws.sc, ws.g);
  launch(k_scale_v0, vec_blocks(ws.n), KT, 0, s, ws.V, ws.n, ws.sc);
  MPDOK_LAUNCH_CHECK("cycle start");
  return MPDOK_OK;
}

// Host copies of a cycle's done flag, two slots per host thread and device
// (pinned, so the copy is asynchronous) with the events that mark them written.
struct DoneProbe {
  int* flag = nullptr;
  cudaEvent_t ev[2] = {nullptr, nullptr};
  bool ok = false;
  DoneProbe() {
    ok = cudaMallocHost(reinterpret_cast<void**>(&flag), 2 * sizeof(int)) == cudaSuccess &&
         cudaEventCreateWithFlags(&ev[0], cudaEventDisableTiming) == cudaSuccess &&
         cudaEventCreateWithFlags(&ev[1], cudaEventDisableTiming) == cudaSuccess;
    if (!ok) cudaGetLastError();
  }
};

int arnoldi_cycle(const KWs& ws, const Operator32& A, int m, int reorth, double tol_rel, const Precond* pc,
                  float* x32, double* x64, cudaStream_t s) {
  const long long n = ws.n;
  const ArnState st = arn_state(ws);
  const size_t smem_dots = (size_t)ws.ch * sizeof(float);
  const size_t smem_apply = (size_t)(KMAX_RESTART + 1 + ws.ch) * sizeof(float);
  // Every kernel of an iteration is predicated on the device done flag, so
  // the cycle may be queued whole; but a predicated-off iteration still costs
  // its launches (~75 us at N = 32768, a preconditioned cycle converges in a
  // few of its 30).  So the host reads the flag two iterations behind the
  // queue (the GPU always has the next iteration queued) and stops queueing
  // once it is set.  Not while the stream is being captured.
  constexpr int MAX_DEV = 64;
  thread_local DoneProbe* probes[MAX_DEV] = {};
  int dev = 0;
  MPDOK_CUDA_TRY(cudaGetDevice(&dev));
  if (dev >= 0 && dev < MAX_DEV && probes[dev] == nullptr) probes[dev] = new DoneProbe();
  DoneProbe* pp = (dev >= 0 && dev < MAX_DEV) ? probes[dev] : nullptr;
  cudaStreamCaptureStatus cap = cudaStreamCaptureStatusNone;
  const bool poll = pp != nullptr && pp->ok && cudaStreamIsCapturing(s, &cap) == cudaSuccess &&
                    cap == cudaStreamCaptureStatusNone;
  for (int k = 0; k < m; ++k) {
    if (poll && k >= 2) {
      MPDOK_CUDA_TRY(cudaEventSynchronize(pp->ev[k & 1]));  // the flag after iteration k - 2
      if (pp->flag[k & 1]) break;
    }
    const float* vk = ws.V + (long long)k * ws.ldv;
    const float* opnd = vk;
    if (pc && pc->apply) {
      float* zk = pc->Z ? pc->Z + (long long)k * pc->ldz : pc->z;
      MPDOK_TRY(pc->apply(pc->ctx, vk, zk, s, &ws.sc->done));
      opnd = zk;
    }
    MPDOK_TRY(A.apply(A.ctx, opnd, ws.w, 1, ws.ldv, s, &ws.sc->done));
    double* Hcol = ws.H + (long long)k * st.ldh;
    launch(k_dots, ws.nblk, KT, smem_dots, s, ws.V, ws.ldv, k + 1, ws.w, n, ws.ch, ws.parts, ws.tickets + 0, Hcol, ws.sc);
    if (reorth >= 2) {
      launch(k_apply<0>, ws.nblk, KT, smem_apply, s, ws.V, ws.ldv, k + 1, ws.w, n, ws.ch, Hcol, ws.parts, ws.tickets + 1,
                                                  ws.h2, Hcol, ws.sc, st, k, tol_rel);
      launch(k_apply<1>, ws.nblk, KT, smem_apply, s, ws.V, ws.ldv, k + 1, ws.w, n, ws.ch, ws.h2, ws.parts,
                                                  ws.tickets + 2, nullptr, nullptr, ws.sc, st, k, tol_rel);
    } else {
      launch(k_apply<1>, ws.nblk, KT, smem_apply, s, ws.V, ws.ldv, k + 1, ws.w, n, ws.ch, Hcol, ws.parts,
                                                  ws.tickets + 2, nullptr, nullptr, ws.sc, st, k, tol_rel);
    }
    launch(k_normalize, vec_blocks(n), KT, 0, s, ws.w, ws.V + (long long)(k + 1) * ws.ldv, n, ws.sc);
    MPDOK_LAUNCH_CHECK("arnoldi step");
    if (poll) {
      MPDOK_CUDA_TRY(cudaMemcpyAsync(&pp->flag[k & 1], &ws.sc->done, sizeof(int), cudaMemcpyDeviceToHost, s));
      MPDOK_CUDA_TRY(cudaEventRecord(pp->ev[k & 1], s));
    }
  }
  launch(k_backsub, 1, 32, 0, s, ws.sc, st);
  if (pc && pc->apply && pc->Z) {
    // x += M^{-1} V y = Z y
    if (x64) launch(k_update<double>, vec_blocks(n), KT, 0, s, (const float*)pc->Z, pc->ldz, ws.y, ws.sc, n, x64, nullptr);
    else launch(k_update<float>, vec_blocks(n), KT, 0, s, (const float*)pc->Z, pc->ldz, ws.y, ws.sc, n, x32, nullptr);
  } else if (pc && pc->apply) {
    // x += M^{-1} (V y): t = V y into w, z = M^{-1} t, x += z.
    launch(k_update<float>, vec_blocks(n), KT, 0, s, ws.V, ws.ldv, ws.y, ws.sc, n, nullptr, ws.w);
    MPDOK_TRY(pc->apply(pc->ctx, ws.w, pc->z, s, nullptr));
    if (x64) launch(k_axpy_f32<double>, vec_blocks(n), KT, 0, s, pc->z, n, x64, ws.sc);
    else launch(k_axpy_f32<float>, vec_blocks(n), KT, 0, s, pc->z, n, x32, ws.sc);
  } else {
    if (x64) launch(k_update<double>, vec_blocks(n), KT, 0, s, ws.V, ws.ldv, ws.y, ws.sc, n, x64, nullptr);
    else launch(k_update<float>, vec_blocks(n), KT, 0, s, ws.V, ws.ldv, ws.y, ws.sc, n, x32, nullptr);
  }
  MPDOK_LAUNCH_CHECK("arnoldi update");
  return MPDOK_OK;
}

static void hist_push(mpdok_solve_info* info, int it, double rel) {
  if (!info) return;
  if (info->n_history < MPDOK_HISTORY_MAX) {
    info->hist_iter[info->n_history] = it;
    info->history[info->n_history] = rel;
    info->n_history++;
  } else {
    info->hist_iter[MPDOK_HISTORY_MAX - 1] = it;
    info->history[MPDOK_HISTORY_MAX - 1] = rel;
  }
  info->relres = rel;
}

static void info_reset(mpdok_solve_info* info) {
  if (info) std::memset(info, 0, sizeof(*info));
}

int ws_prepare(const KWs& ws, size_t work_bytes, cudaStream_t s) {
  MPDOK_ARG_CHECK(ws.V != nullptr, "null workspace");
  if (work_bytes < ws.total) {
    set_error("invalid argument: Krylov workspace too small (%zu < %zu bytes)", work_bytes, ws.total);
    return MPDOK_ERR_INVALID_ARG;
  }
  MPDOK_CUDA_TRY(cudaMemsetAsync(ws.tickets, 0, sizeof(unsigned) * 8, s));
  MPDOK_CUDA_TRY(cudaMemsetAsync(ws.sc, 0, sizeof(KScal), s));
  return MPDOK_OK;
}

int fp64_residual(const KWs& ws, const Residual64& R, const double* b, const double* x, KScal* hs, cudaStream_t s) {
  MPDOK_TRY(R.apply(R.ctx, b, x, ws.r64, &ws.sc->nrm2, 1, ws.ldv, s));
  return read_scal(ws, hs, s);
}

static int host_bnorm(const KWs& ws, const double* b, double* bnorm, cudaStream_t s) {
  MPDOK_TRY(norm2_f64(ws, b, ws.n, &ws.sc->aux, s));
  KScal hs;
  MPDOK_TRY(read_scal(ws, &hs, s));
  *bnorm = std::sqrt(hs.aux);
  if (!std::isfinite(*bnorm)) {
    set_error("the right-hand side has non-finite entries");
    return MPDOK_ERR_NONFINITE;
  }
  return MPDOK_OK;
}

// Restarted FP32 GMRES on rhs64 (dense_krylov.py:212-331); x64 in/out.
int gmres_core(const KWs& ws, const Operator32& A, const Residual64& R, const double* rhs64, double* x64, double tol,
               int maxiter, int restart, mpdok_solve_info* info, cudaStream_t s) {
  const long long n = ws.n;
  if (maxiter <= 0) maxiter = (int)std::min<long long>(n, INT32_MAX);
  double bnorm = 0.0;
  MPDOK_TRY(host_bnorm(ws, rhs64, &bnorm, s));
  if (info) info->bnorm = bnorm;
  if (bnorm == 0.0) {
    MPDOK_CUDA_TRY(cudaMemsetAsync(x64, 0, sizeof(double) * n, s));
    hist_push(info, 0, 0.0);
    if (info) info->converged = 1;
    return MPDOK_OK;
  }
  MPDOK_TRY(convert_any(rhs64, MPDOK_F64, ws.b32, MPDOK_F32, n, s));
  MPDOK_TRY(convert_any(x64, MPDOK_F64, ws.x32, MPDOK_F32, n, s));
  int total = 0;
  bool converged = false;
  double prev = std::numeric_limits<double>::infinity();
  const int max_restarts = (maxiter + restart - 1) / restart;
  KScal hs;
  for (int outer = 0; outer < max_restarts; ++outer) {
    // r = b32 - A32 x32 (FP32), start vector of the cycle.
    MPDOK_TRY(A.apply(A.ctx, ws.x32, ws.w, 1, ws.ldv, s, nullptr));
    launch(k_sub_from, vec_blocks(n), KT, 0, s, (const float*)ws.b32, ws.w, n);
    MPDOK_TRY(cycle_start_from_f32(ws, ws.w, s));
    MPDOK_TRY(read_scal(ws, &hs, s));
    if (hs.beta == 0.0) { converged = true; break; }
    const int mm = std::min(restart, maxiter - total);
    if (mm <= 0) break;
    MPDOK_TRY(arnoldi_cycle(ws, A, mm, 1, 0.0, nullptr, ws.x32, nullptr, s));
    MPDOK_TRY(convert_any(ws.x32, MPDOK_F32, ws.x64t, MPDOK_F64, n, s));
    MPDOK_TRY(fp64_residual(ws, R, rhs64, ws.x64t, &hs, s));
    total += hs.m_used;
    const double rel = std::sqrt(hs.nrm2) / bnorm;
    hist_push(info, total, rel);
    if (info) { info->outer_iters++; info->inner_iters = total; }
    if (!std::isfinite(rel)) { set_error("GMRES: non-finite residual"); return MPDOK_ERR_NONFINITE; }
    if (rel < tol) { converged = true; break; }
    if (rel > prev * (1.0 - 1e-2)) { if (info) info->stagnated = 1; break; }
    prev = rel;
  }
  MPDOK_TRY(convert_any(ws.x32, MPDOK_F32, x64, MPDOK_F64, n, s));
  if (info) info->converged = converged ? 1 : 0;
  return MPDOK_OK;
}

int gmres_ir_core(const KWs& ws, const Operator32& A, const Residual64& R, const double* b, double* x, double tol,
                  int maxiter_outer, int restart, double inner_tol, const Precond* pc, mpdok_solve_info* info,
                  cudaStream_t s, double* xbest) {
  const long long n = ws.n;
  // ||b|| and ||x0|| in one host read; from x0 = 0 the first residual is b
  // itself, which saves one full FP64 product (8 N^2 bytes, or an N^2
  // matrix-free evaluation)
  MPDOK_TRY(norm2_f64(ws, b, n, &ws.sc->aux, s));
  MPDOK_TRY(norm2_f64(ws, x, n, &ws.sc->alpha, s));
  KScal h0;
  MPDOK_TRY(read_scal(ws, &h0, s));
  const double bnorm = std::sqrt(h0.aux);
  const bool x_zero = h0.alpha == 0.0;
  if (info) info->bnorm = bnorm;
  if (!std::isfinite(bnorm) || !std::isfinite(h0.alpha)) {
    set_error("GMRES-IR: the right-hand side or the initial guess has non-finite entries");
    return MPDOK_ERR_NONFINITE;
  }
  if (bnorm == 0.0) {
    MPDOK_CUDA_TRY(cudaMemsetAsync(x, 0, sizeof(double) * n, s));
    hist_push(info, 0, 0.0);
    if (info) info->converged = 1;
    return MPDOK_OK;
  }
  bool converged = false, diverged = false;
  double best = INFINITY;
  KScal hs;
  int inner_total = 0;
  // guarded mode (xbest != nullptr): keep the best iterate; a non-finite
  // residual or one 1e3 x above the best ends the solve with the best restored
  auto guard = [&](double rel, int it) -> int {
    if (!std::isfinite(rel) || rel > 1e3 * best) {
      MPDOK_CUDA_TRY(cudaMemcpyAsync(x, xbest, sizeof(double) * n, cudaMemcpyDeviceToDevice, s));
      hist_push(info, it, best);
      diverged = true;
    } else if (rel < best) {
      best = rel;
      MPDOK_CUDA_TRY(cudaMemcpyAsync(xbest, x, sizeof(double) * n, cudaMemcpyDeviceToDevice, s));
    }
    return MPDOK_OK;
  };
  for (int outer = 0; outer < maxiter_outer; ++outer) {
    double rel;
    if (outer == 0 && x_zero) {
      MPDOK_CUDA_TRY(cudaMemcpyAsync(ws.r64, b, sizeof(double) * n, cudaMemcpyDeviceToDevice, s));
      rel = 1.0;  // ||b - A 0|| / ||b||
    } else {
      MPDOK_TRY(fp64_residual(ws, R, b, x, &hs, s));
      if (outer > 0) inner_total += hs.m_used;
      rel = std::sqrt(hs.nrm2) / bnorm;
    }
    hist_push(info, outer, rel);
    if (xbest) {
      MPDOK_TRY(guard(rel, outer));
      if (diverged) break;
    } else if (!std::isfinite(rel)) {
      set_error("GMRES-IR: non-finite residual");
      return MPDOK_ERR_NONFINITE;
    }
    if (rel < tol) { converged = true; break; }
    MPDOK_TRY(cycle_start_from_f64(ws, ws.r64, s));
    MPDOK_TRY(arnoldi_cycle(ws, A, restart, 2, inner_tol, pc, nullptr, x, s));
    if (info) info->outer_iters = outer + 1;
  }
  if (!converged && !diverged) {
    MPDOK_TRY(fp64_residual(ws, R, b, x, &hs, s));
    if (maxiter_outer > 0) inner_total += hs.m_used;
    const double rel = std::sqrt(hs.nrm2) / bnorm;
    hist_push(info, maxiter_outer, rel);
    if (xbest) {
      MPDOK_TRY(guard(rel, maxiter_outer));
      if (!diverged && rel > best) {  // an earlier iterate was better
        MPDOK_CUDA_TRY(cudaMemcpyAsync(x, xbest, sizeof(double) * n, cudaMemcpyDeviceToDevice, s));
        hist_push(info, maxiter_outer, best);
      }
    }
    converged = info ? info->relres < tol : rel < tol;
  }
  if (info) {
    info->converged = converged ? 1 : 0;
    info->inner_iters = inner_total;
    if (diverged) info->stagnated = 2;
  }
  return MPDOK_OK;
}

int dense_gmres_ir_core(const KWs& ws, const Operator32& A, const Residual64& R, const double* b, double* x,
                        double tol, int maxiter_outer, int restart, int maxiter_inner, mpdok_solve_info* info,
                        cudaStream_t s) {
  const long long n = ws.n;
  double bnorm = 0.0;
  MPDOK_TRY(host_bnorm(ws, b, &bnorm, s));
  if (info) info->bnorm = bnorm;
  if (bnorm == 0.0) {
    MPDOK_CUDA_TRY(cudaMemsetAsync(x, 0, sizeof(double) * n, s));
    hist_push(info, 0, 0.0);
    if (info) info->converged = 1;
    return MPDOK_OK;
  }
  MPDOK_CUDA_TRY(cudaMemsetAsync(x, 0, sizeof(double) * n, s));
  double* rhs = ws.e64 + ws.ldv;  // second FP64 vector of the e64 pair
  bool converged = false;
  KScal hs;
  int inner_total = 0;
  for (int outer = 0; outer < maxiter_outer; ++outer) {
    MPDOK_TRY(fp64_residual(ws, R, b, x, &hs, s));
    const double rel = std::sqrt(hs.nrm2) / bnorm;
    hist_push(info, outer, rel);
    if (!std::isfinite(rel)) { set_error("GMRES-IR: non-finite residual"); return MPDOK_ERR_NONFINITE; }
    if (rel < tol) { converged = true; break; }
    MPDOK_CUDA_TRY(cudaMemcpyAsync(rhs, ws.r64, sizeof(double) * n, cudaMemcpyDeviceToDevice, s));
    MPDOK_CUDA_TRY(cudaMemsetAsync(ws.e64, 0, sizeof(double) * n, s));
    mpdok_solve_info inner;
    info_reset(&inner);
    MPDOK_TRY(gmres_core(ws, A, R, rhs, ws.e64, 1e-6, maxiter_inner, restart, &inner, s));
    inner_total += inner.inner_iters;
    launch(k_axpy_f64, vec_blocks(n), KT, 0, s, (const double*)ws.e64, x, n);
    MPDOK_LAUNCH_CHECK("gmres_ir update");
    if (info) info->outer_iters = outer + 1;
  }
  MPDOK_TRY(fp64_residual(ws, R, b, x, &hs, s));
  const double rel = std::sqrt(hs.nrm2) / bnorm;
  hist_push(info, maxiter_outer, rel);
  converged = converged || rel < tol;
  if (info) { info->converged = converged ? 1 : 0; info->inner_iters = inner_total; }
  return MPDOK_OK;
}

int cg_core(const KWs& ws, const Operator32& A, const Residual64& R, const double* b, double* x, double tol,
            int maxiter, int check_every, mpdok_solve_info* info, cudaStream_t s) {
  const long long n = ws.n;
  if (maxiter < 0) maxiter = (int)std::min<long long>(n, INT32_MAX);
  double bnorm = 0.0;
  MPDOK_TRY(host_bnorm(ws, b, &bnorm, s));
  if (info) info->bnorm = bnorm;
  if (bnorm == 0.0) {
    MPDOK_CUDA_TRY(cudaMemsetAsync(x, 0, sizeof(double) * n, s));
    hist_push(info, 0, 0.0);
    if (info) info->converged = 1;
    return MPDOK_OK;
  }
  float* xr = ws.x32;
  float* r = ws.w;
  float* p = ws.p32;
  float* q = ws.q32;
  MPDOK_TRY(convert_any(b, MPDOK_F64, ws.b32, MPDOK_F32, n, s));
  MPDOK_TRY(convert_any(x, MPDOK_F64, xr, MPDOK_F32, n, s));
  MPDOK_TRY(A.apply(A.ctx, xr, r, 1, ws.ldv, s, nullptr));
  launch(k_sub_from, vec_blocks(n), KT, 0, s, (const float*)ws.b32, r, n);
  launch(k_norm2<float>, vec_blocks(n), KT, 0, s, (const float*)r, n, ws.parts, ws.tickets + 4, &ws.sc->nrm2);
  MPDOK_CUDA_TRY(cudaMemcpyAsync(p, r, sizeof(float) * n, cudaMemcpyDeviceToDevice, s));
  launch(k_set_rs, 1, 32, 0, s, ws.sc);
  bool converged = false;
  double prev = std::numeric_limits<double>::infinity();
  KScal hs;
  int last_k = -1;
  int it_done = 0;
  for (int k = 0; k < maxiter; ++k) {
    last_k = k;
    if (k % check_every == 0) {
      MPDOK_TRY(convert_any(xr, MPDOK_F32, ws.x64t, MPDOK_F64, n, s));
      MPDOK_TRY(fp64_residual(ws, R, b, ws.x64t, &hs, s));
      const double rel = std::sqrt(hs.nrm2) / bnorm;
      hist_push(info, k, rel);
      if (info) info->outer_iters++;
      if (!std::isfinite(rel)) { set_error("CG: non-finite residual"); return MPDOK_ERR_NONFINITE; }
      if (rel < tol) { converged = true; break; }
      if (rel > prev * (1.0 - 1e-2)) { if (info) info->stagnated = 1; break; }
      prev = rel;
      if (hs.done) break;  // p.Ap == 0: nothing more to do
    }
    MPDOK_TRY(A.apply(A.ctx, p, q, 1, ws.ldv, s, &ws.sc->done));
    launch(k_cg_pap, vec_blocks(n), KT, 0, s, (const float*)p, (const float*)q, n, ws.parts, ws.tickets + 0, ws.sc);
    launch(k_cg_xr, vec_blocks(n), KT, 0, s, xr, r, (const float*)p, (const float*)q, n, ws.parts, ws.tickets + 1,
           ws.sc);
    launch(k_cg_p, vec_blocks(n), KT, 0, s, p, (const float*)r, n, (const KScal*)ws.sc);
    MPDOK_LAUNCH_CHECK("cg iteration");
    it_done = k + 1;
  }
  if (!converged) {
    MPDOK_TRY(convert_any(xr, MPDOK_F32, ws.x64t, MPDOK_F64, n, s));
    MPDOK_TRY(fp64_residual(ws, R, b, ws.x64t, &hs, s));
    const double rel = std::sqrt(hs.nrm2) / bnorm;
    hist_push(info, last_k + 1, rel);
    converged = rel < tol;
  }
  MPDOK_TRY(convert_any(xr, MPDOK_F32, x, MPDOK_F64, n, s));
  if (info) { info->converged = converged ? 1 : 0; info->inner_iters = it_done; }
  return MPDOK_OK;
}

CgIrWs cgir_layout(long long n, int K, void* base) {
  CgIrWs w;
  w.n = n;
  w.K = K;
  w.ld = (long long)align_up((size_t)std::max(1LL, n), 64);
  w.nblk = vec_blocks(n);
  size_t off = 0;
  auto take = [&](size_t b) { size_t o = off; off = align_up(off + b, 256); return o; };
  const size_t fcol = (size_t)w.ld * K * sizeof(float);
  const size_t dcol = (size_t)w.ld * K * sizeof(double);
  size_t oR = take(dcol), oB = take(dcol), oX = take(dcol), oE = take(fcol), or_ = take(fcol), op = take(fcol),
         oq = take(fcol), oz = take(fcol);
  size_t oparts = take(sizeof(double) * (size_t)w.nblk * K + 64);
  size_t ocols = take(sizeof(MColState) * K);
  size_t og = take(64);
  size_t onrm = take(sizeof(double) * K);
  size_t otk = take(64);
  w.total = off;
  if (base) {
    char* b = (char*)base;
    w.R64 = (double*)(b + oR); w.B64 = (double*)(b + oB); w.X64 = (double*)(b + oX);
    w.E = (float*)(b + oE); w.r = (float*)(b + or_); w.p = (float*)(b + op); w.q = (float*)(b + oq);
    w.z = (float*)(b + oz);
    w.parts = (double*)(b + oparts); w.cols = (void*)(b + ocols); w.g = (void*)(b + og);
    w.nrm2 = (double*)(b + onrm); w.ticket = (unsigned*)(b + otk);
  }
  return w;
}

int cg_ir_core(const CgIrWs& w, const Operator32& A, const Residual64& R, const double* B, long long ldb, double* X,
               long long ldx, double tol, int maxiter_outer, double inner_tol, int inner_maxiter, const Precond* pc,
               mpdok_solve_info* info, cudaStream_t s) {
  const long long n = w.n;
  const int K = w.K;
  const long long ld = w.ld;
  MColState* cols = (MColState*)w.cols;
  MCGGlobal* g = (MCGGlobal*)w.g;
  dim3 grid(w.nblk, K);
  MPDOK_CUDA_TRY(cudaMemsetAsync(w.ticket, 0, 64, s));
  MPDOK_CUDA_TRY(cudaMemsetAsync(w.X64, 0, sizeof(double) * ld * K, s));
  launch(k_copy_cols, grid, KT, 0, s, B, ldb, w.B64, ld, n);
  // ||B_j||
  MPDOK_TRY(colnorms_f64(w.B64, n, K, ld, w.nrm2, s));
  std::vector<double> bn(K), rn(K);
  MPDOK_CUDA_TRY(cudaMemcpyAsync(bn.data(), w.nrm2, sizeof(double) * K, cudaMemcpyDeviceToHost, s));
  MPDOK_CUDA_TRY(cudaStreamSynchronize(s));
  for (int j = 0; j < K; ++j) {
    bn[j] = std::sqrt(bn[j]);  // colnorms_f64 returns squared norms
    if (!std::isfinite(bn[j])) {
      set_error("CG-IR: right-hand side %d has non-finite entries", j);
      return MPDOK_ERR_NONFINITE;
    }
  }
  if (info) info->bnorm = *std::max_element(bn.begin(), bn.end());
  bool converged = false;
  int inner_total = 0;
  for (int outer = 0; outer <= maxiter_outer; ++outer) {
    MPDOK_TRY(R.apply(R.ctx, w.B64, w.X64, w.R64, w.nrm2, K, ld, s));
    MPDOK_CUDA_TRY(cudaMemcpyAsync(rn.data(), w.nrm2, sizeof(double) * K, cudaMemcpyDeviceToHost, s));
    MPDOK_CUDA_TRY(cudaStreamSynchronize(s));
    double worst = 0.0;
    for (int j = 0; j < K; ++j) {
      const double rel = bn[j] > 0 ? std::sqrt(rn[j]) / bn[j] : 0.0;
      worst = std::max(worst, rel);
    }
    hist_push(info, outer, worst);
    if (!std::isfinite(worst)) { set_error("CG-IR: non-finite residual"); return MPDOK_ERR_NONFINITE; }
    if (worst < tol) { converged = true; break; }
    if (outer == maxiter_outer) break;
    // inner FP32 CG on A E = R, all columns in lockstep
    launch(k_mcg_init, grid, KT, 0, s, (const double*)w.R64, ld, n, w.E, w.r, w.p, w.parts, w.ticket, cols, g);
    if (pc) {
      // z = M^-1 r, p = z, rz = r . z
      if (pc->apply_cols) {
        MPDOK_TRY(pc->apply_cols(pc->ctx, w.r, w.z, K, ld, s));
      } else {
        for (int c = 0; c < K; ++c)
          MPDOK_TRY(pc->apply(pc->ctx, w.r + (long long)c * ld, w.z + (long long)c * ld, s, nullptr));
      }
      launch(k_mcg_rz, grid, KT, 0, s, (const float*)w.r, (const float*)w.z, ld, n, w.parts, w.ticket + 3, cols,
             (const MCGGlobal*)g, 1);
      MPDOK_CUDA_TRY(cudaMemcpyAsync(w.p, w.z, sizeof(float) * ld * K, cudaMemcpyDeviceToDevice, s));
    }
    MCGGlobal hg{0, 0};
    int it = 0;
    while (it < inner_maxiter) {
      const int batch = std::min(20, inner_maxiter - it);
      for (int b = 0; b < batch; ++b) {
        MPDOK_TRY(A.apply(A.ctx, w.p, w.q, K, ld, s, &g->done));
        launch(k_mcg_pap, grid, KT, 0, s, (const float*)w.p, (const float*)w.q, ld, n, w.parts, w.ticket + 1, cols,
               (const MCGGlobal*)g);
        launch(k_mcg_xr, grid, KT, 0, s, w.E, w.r, (const float*)w.p, (const float*)w.q, ld, n, w.parts,
               w.ticket + 2, cols, g, inner_tol, pc ? 1 : 0);
        if (pc) {
          if (pc->apply_cols) {
            MPDOK_TRY(pc->apply_cols(pc->ctx, w.r, w.z, K, ld, s));
          } else {
            for (int c = 0; c < K; ++c)
              MPDOK_TRY(pc->apply(pc->ctx, w.r + (long long)c * ld, w.z + (long long)c * ld, s, &g->done));
          }
          launch(k_mcg_rz, grid, KT, 0, s, (const float*)w.r, (const float*)w.z, ld, n, w.parts, w.ticket + 3, cols,
                 (const MCGGlobal*)g, 0);
        }
        launch(k_mcg_p, grid, KT, 0, s, w.p, (const float*)(pc ? w.z : w.r), ld, n, (const MColState*)cols,
               (const MCGGlobal*)g);
      }
      MPDOK_LAUNCH_CHECK("cg-ir inner");
      it += batch;
      MPDOK_CUDA_TRY(cudaMemcpyAsync(&hg, g, sizeof(hg), cudaMemcpyDeviceToHost, s));
      MPDOK_CUDA_TRY(cudaStreamSynchronize(s));
      if (hg.done) break;
    }
    inner_total += hg.iters;
    launch(k_add_cols, grid, KT, 0, s, (const float*)w.E, ld, w.X64, ld, n);
    MPDOK_LAUNCH_CHECK("cg-ir update");
    if (info) info->outer_iters = outer + 1;
  }
  launch(k_copy_cols, grid, KT, 0, s, (const double*)w.X64, ld, X, ldx, n);
  MPDOK_LAUNCH_CHECK("cg-ir out");
  if (info) {
    info->converged = converged ? 1 : 0;
    info->inner_iters = inner_total;
  }
  return MPDOK_OK;
}

}  // namespace mpdok

using namespace mpdok;

extern "C" size_t mpdok_krylov_workspace_size(long long n, int restart) {
  if (n < 0 || restart < 1) return 0;
  return krylov_layout(n, std::min(restart, KMAX_RESTART), nullptr).total;
}

static StoredCtx make_stored(const KWs& ws, const float* A32, long long lda32, const double* A64, long long lda) {
  StoredCtx c;
  c.A32 = A32;
  c.lda32 = lda32;
  c.A64 = A64;
  c.lda64 = lda;
  c.n = ws.n;
  c.gw = ws.gw;
  c.gbytes = ws.gbytes;
  return c;
}

extern "C" int mpdok_gmres_ir(const double* A64, long long lda, float* A32, long long lda32, int a32_ready,
                              long long n, const double* b, double* x, double tol, int maxiter_outer, int restart,
                              double inner_tol, void* work, size_t work_bytes, mpdok_solve_info* info,
                              cudaStream_t s) {
  info_reset(info);
  MPDOK_ARG_CHECK(n >= 0, "negative n");
  MPDOK_ARG_CHECK(restart >= 1 && restart <= KMAX_RESTART, "restart must be in [1, 1024]");
  MPDOK_ARG_CHECK(maxiter_outer >= 0, "negative maxiter_outer");
  if (n == 0) { if (info) info->converged = 1; return MPDOK_OK; }
  MPDOK_ARG_CHECK(A64 && A32 && b && x, "null pointer");
  MPDOK_ARG_CHECK(lda >= n && lda32 >= n, "lda < n");
  KWs ws = krylov_layout(n, restart, work);
  MPDOK_TRY(ws_prepare(ws, work_bytes, s));
  if (!a32_ready) MPDOK_TRY(convert_matrix_f64_f32(A64, lda, A32, lda32, n, n, s));
  StoredCtx c = make_stored(ws, A32, lda32, A64, lda);
  return gmres_ir_core(ws, stored_op32(&c), stored_res64(&c), b, x, tol, maxiter_outer, restart, inner_tol, nullptr,
                       info, s);
}

extern "C" int mpdok_gmres(const float* A32, long long lda32, const double* A64, long long lda, long long n,
                           const double* b, double* x, double tol, int maxiter, int restart, void* work,
                           size_t work_bytes, mpdok_solve_info* info, cudaStream_t s) {
  info_reset(info);
  MPDOK_ARG_CHECK(n >= 0, "negative n");
  MPDOK_ARG_CHECK(restart >= 1 && restart <= KMAX_RESTART, "restart must be in [1, 1024]");
  if (n == 0) { if (info) info->converged = 1; return MPDOK_OK; }
  MPDOK_ARG_CHECK(A32 && A64 && b && x, "null pointer (GMRES needs the FP64 matrix for residual checks)");
  KWs ws = krylov_layout(n, restart, work);
  MPDOK_TRY(ws_prepare(ws, work_bytes, s));
  StoredCtx c = make_stored(ws, A32, lda32, A64, lda);
  return gmres_core(ws, stored_op32(&c), stored_res64(&c), b, x, tol, maxiter, restart, info, s);
}

extern "C" int mpdok_dense_gmres_ir(const float* A32, long long lda32, const double* A64, long long lda, long long n,
                                    const double* b, double* x, double tol, int maxiter_outer, int restart,
                                    int maxiter_inner, void* work, size_t work_bytes, mpdok_solve_info* info,
                                    cudaStream_t s) {
  info_reset(info);
  MPDOK_ARG_CHECK(n >= 0, "negative n");
  MPDOK_ARG_CHECK(restart >= 1 && restart <= KMAX_RESTART, "restart must be in [1, 1024]");
  if (n == 0) { if (info) info->converged = 1; return MPDOK_OK; }
  MPDOK_ARG_CHECK(A32 && A64 && b && x, "null pointer");
  KWs ws = krylov_layout(n, restart, work);
  MPDOK_TRY(ws_prepare(ws, work_bytes, s));
  StoredCtx c = make_stored(ws, A32, lda32, A64, lda);
  return dense_gmres_ir_core(ws, stored_op32(&c), stored_res64(&c), b, x, tol, maxiter_outer, restart, maxiter_inner,
                             info, s);
}

extern "C" int mpdok_cg(const float* A32, long long lda32, const double* A64, long long lda, long long n,
                        const double* b, double* x, double tol, int maxiter, int check_every, void* work,
                        size_t work_bytes, mpdok_solve_info* info, cudaStream_t s) {
  info_reset(info);
  MPDOK_ARG_CHECK(n >= 0, "negative n");
  MPDOK_ARG_CHECK(check_every >= 1, "check_every must be >= 1");
  if (n == 0) { if (info) info->converged = 1; return MPDOK_OK; }
  MPDOK_ARG_CHECK(A32 && A64 && b && x, "null pointer (CG needs the FP64 matrix for residual checks)");
  KWs ws = krylov_layout(n, 1, work);
  MPDOK_TRY(ws_prepare(ws, work_bytes, s));
  StoredCtx c = make_stored(ws, A32, lda32, A64, lda);
  return cg_core(ws, stored_op32(&c), stored_res64(&c), b, x, tol, maxiter, check_every, info, s);
}
