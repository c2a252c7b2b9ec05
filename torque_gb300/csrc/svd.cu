// Block-level truncated SVD and QR of a block-sparse tensor (the step after
// the contraction in PEPS / MPS sweeps; the reference has only a cuSOLVER QR
// example that nothing calls, test/cusolver_playground.cpp:7).
//
// The legs are split into row legs (given) and column legs (the rest, in
// order).  Every block is a box of a row-leg box X and a column-leg box Y; the
// X and Y linked through blocks form connected classes (for a charge-conserving
// tensor, one class per charge sector), and the tensor is block diagonal over
// them: one dense matrix per class (its X stacked as rows, its Y as columns,
// absent blocks zero).  Each class matrix is decomposed on the device by
// one-sided Jacobi rotations (Hestenes; high relative accuracy, FP64), one CTA
// per class; the singular values of all classes are ranked together and the
// largest are kept (at most max_keep, and above cutoff times the largest).
// The factors come back as block-sparse tensors over a new bond leg with one
// sector per class that keeps a value:
//   U[row legs..., bond], S[bond] (the values, descending in each sector),
//   V[bond, column legs...], with T ~ sum_k U[..., k] S[k] V[k, ...].
#include <algorithm>
#include <cmath>
#include <cstring>
#include <map>
#include <numeric>
#include <vector>

#include "tq_internal.h"

namespace tq {

static inline unsigned blocks_of(int64_t n) { return (unsigned)((n + 255) / 256); }

// One element per thread: the class matrix (rows = row-leg index within the
// class, columns = column-leg index, column-major with leading dimension ld;
// transposed for classes with fewer rows than columns) receives the block's
// elements.  Per block: class matrix base, row and column offsets of its X and
// Y in the class, leading dimension, orientation.
struct SvdBlock {
  int64_t base, row0, col0, ld;
  int32_t transposed, pad;
};

__global__ void svd_gather_kernel(DevBS T, int32_t nr, const int32_t *rl, int32_t nc,
                                  const int32_t *cl, const SvdBlock *sb, const int64_t *estart,
                                  int64_t ne, double *mat) {
  const int64_t g = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (g >= ne) return;
  int64_t lo = 0, hi = T.nb - 1;
  while (lo < hi) {
    const int64_t mid = (lo + hi + 1) >> 1;
    if (estart[mid] <= g) lo = mid; else hi = mid - 1;
  }
  const int64_t b = lo;
  int64_t e = g - estart[b];
  const int32_t r = T.rank;
  const int64_t *bb = T.begin + b * r, *be = T.end + b * r, *st = T.strides + b * r;
  int64_t x[TQ_MAXR];
  for (int l = 0; l < r; l++) {
    const int64_t d = be[l] - bb[l] + 1;
    x[l] = e % d;
    e /= d;
  }
  int64_t addr = T.offsets[b], row = 0, col = 0, m = 1;
  for (int l = 0; l < r; l++) addr += x[l] * st[l];
  for (int q = 0; q < nr; q++) {
    row += x[rl[q]] * m;
    m *= be[rl[q]] - bb[rl[q]] + 1;
  }
  m = 1;
  for (int q = 0; q < nc; q++) {
    col += x[cl[q]] * m;
    m *= be[cl[q]] - bb[cl[q]] + 1;
  }
  const SvdBlock s = sb[b];
  const int64_t i = s.row0 + row, j = s.col0 + col;
  const int64_t at = s.transposed ? s.base + j + i * s.ld : s.base + i + j * s.ld;
  atomicAdd(mat + at, ((const double *)T.data)[addr]);
}

struct SvdClass {
  int64_t a, v;   // class matrix (m x n, ld m) and its right factor (n x n) in scratch
  int32_t m, n;   // after orientation: m >= n
  int32_t sweeps, pad;
};

// Hestenes one-sided Jacobi on one class (one CTA): A <- A J, V <- V J until
// every column pair is orthogonal to 1e-15 relative; then the singular values
// are the column norms.  Pairs meet in round-robin order (n' = n rounded up to
// even; a pair with a padding column is skipped); each warp rotates one pair
// at a time, its lanes striding over the rows.
__global__ void __launch_bounds__(512) svd_jacobi_kernel(const SvdClass *cls, double *scr,
                                                         double *sigma, const int64_t *sig_off,
                                                         int32_t max_sweeps, int32_t *info) {
  const SvdClass C = cls[blockIdx.x];
  double *A = scr + C.a, *V = scr + C.v;
  const int m = C.m, n = C.n, np = n + (n & 1);
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31, nw = blockDim.x >> 5;
  __shared__ int rotated;
  for (int64_t k = threadIdx.x; k < (int64_t)n * n; k += blockDim.x)
    V[k] = (k % n) == (k / n) ? 1.0 : 0.0;
  __syncthreads();
  int sweep = 0;
  for (; sweep < max_sweeps; sweep++) {
    if (threadIdx.x == 0) rotated = 0;
    __syncthreads();
    for (int round = 0; round < np - 1; round++) {
      for (int pi = warp; pi < np / 2; pi += nw) {
        auto who = [&](int k) { return k == 0 ? 0 : ((k - 1 + round) % (np - 1)) + 1; };
        int p = who(pi), q = who(np - 1 - pi);
        if (p >= n || q >= n) continue;
        if (p > q) { const int t = p; p = q; q = t; }
        double *ap = A + (int64_t)p * m, *aq = A + (int64_t)q * m;
        double al = 0, be = 0, ga = 0;
        for (int i = lane; i < m; i += 32) {
          al += ap[i] * ap[i];
          be += aq[i] * aq[i];
          ga += ap[i] * aq[i];
        }
        for (int o = 16; o; o >>= 1) {
          al += __shfl_xor_sync(0xffffffffu, al, o);
          be += __shfl_xor_sync(0xffffffffu, be, o);
          ga += __shfl_xor_sync(0xffffffffu, ga, o);
        }
        if (fabs(ga) <= 1e-15 * sqrt(al * be) || ga == 0.0) continue;
        const double zeta = (be - al) / (2.0 * ga);
        const double t = (zeta >= 0 ? 1.0 : -1.0) / (fabs(zeta) + sqrt(1.0 + zeta * zeta));
        const double c = 1.0 / sqrt(1.0 + t * t), s = c * t;
        for (int i = lane; i < m; i += 32) {
          const double x = ap[i], y = aq[i];
          ap[i] = c * x - s * y;
          aq[i] = s * x + c * y;
        }
        double *vp = V + (int64_t)p * n, *vq = V + (int64_t)q * n;
        for (int i = lane; i < n; i += 32) {
          const double x = vp[i], y = vq[i];
          vp[i] = c * x - s * y;
          vq[i] = s * x + c * y;
        }
        if (lane == 0) rotated = 1;
      }
      __syncthreads();
    }
    const int any = rotated;
    __syncthreads();
    if (!any) break;
  }
  if (threadIdx.x == 0 && sweep == max_sweeps) atomicOr(info, 1);  // did not converge
  // singular values: column norms; U columns normalised in place
  for (int j = warp; j < n; j += nw) {
    double *aj = A + (int64_t)j * m;
    double s2 = 0;
    for (int i = lane; i < m; i += 32) s2 += aj[i] * aj[i];
    for (int o = 16; o; o >>= 1) s2 += __shfl_xor_sync(0xffffffffu, s2, o);
    const double sg = sqrt(s2);
    const double inv = sg > 0 ? 1.0 / sg : 0.0;
    for (int i = lane; i < m; i += 32) aj[i] *= inv;
    if (lane == 0) sigma[sig_off[blockIdx.x] + j] = sg;
  }
}

// Output scatter: one element per thread of the factor blocks.  Kind 0: U
// block (rows of X x kept columns), 1: V block (kept x columns of Y), 2: S.
struct SvdOut {
  int64_t dst;     // offset in the output tensor's data
  int64_t a, v;    // class scratch (after orientation)
  int64_t sig;     // class singular values
  int64_t perm;    // class column order (descending values) in perm[]
  int32_t m, n;    // class dims after orientation
  int32_t kind, transposed;
  int32_t off, len;  // row (U) or column (V) offset of X / Y in the class, its size
  int32_t keep, pad;
};

__global__ void svd_scatter_kernel(const SvdOut *ob, const int64_t *ostart, int64_t nob,
                                   int64_t ne, const double *scr, const double *sigma,
                                   const int32_t *perm, double *U, double *S, double *V) {
  const int64_t g = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (g >= ne) return;
  int64_t lo = 0, hi = nob - 1;
  while (lo < hi) {
    const int64_t mid = (lo + hi + 1) >> 1;
    if (ostart[mid] <= g) lo = mid; else hi = mid - 1;
  }
  const SvdOut o = ob[lo];
  const int64_t e = g - ostart[lo];
  const int32_t *pc = perm + o.perm;
  if (o.kind == 2) {
    S[o.dst + e] = sigma[o.sig + pc[e]];
    return;
  }
  // left factor of the class: A's columns (not transposed) or V (transposed)
  if (o.kind == 0) {  // U block: element (row r of X, kept k), column-major
    const int64_t r = e % o.len, k = e / o.len;
    const int64_t row = o.off + r, j = pc[k];
    U[o.dst + e] = o.transposed ? scr[o.v + row + j * (int64_t)o.n]
                                : scr[o.a + row + j * (int64_t)o.m];
  } else {  // V block: element (kept k, column c of Y), column-major over (bond, Y)
    const int64_t k = e % o.keep, c = e / o.keep;
    const int64_t col = o.off + c, j = pc[k];
    V[o.dst + e] = o.transposed ? scr[o.a + col + j * (int64_t)o.m]
                                : scr[o.v + col + j * (int64_t)o.n];
  }
}


// ---------------------------------------------------------------- QR
// Householder QR of one class per CTA (FP64): A (m x n, ld m) becomes R in
// its upper triangle and the reflector vectors below it (v_j(j) = 1 implied),
// tau[j] their factors; Q (m x k, k = min(m, n)) is formed by applying the
// reflectors to the first k columns of the identity in reverse order.  The
// signs are then chosen so that R's diagonal is non-negative (the QR of a
// full-rank matrix is then unique).
struct QrClass {
  int64_t a, q, t;  // class matrix, Q, tau (scratch offsets)
  int32_t m, n;
};

__device__ double qr_block_sum(double v, double *red) {
  for (int o = 16; o; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31, nw = blockDim.x >> 5;
  __syncthreads();  // red may still be read by the previous call
  if (lane == 0) red[warp] = v;
  __syncthreads();
  double t = 0;
  for (int w = 0; w < nw; w++) t += red[w];
  return t;
}

// H_j applied to columns c0 .. c1-1 of X (rows j .. m-1, ld m): warp per column
__device__ void qr_apply(const double *A, int64_t m, int j, double tau, double *X, int c0, int c1) {
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31, nw = blockDim.x >> 5;
  const double *v = A + (int64_t)j * m;  // v(j) = 1, v(i > j) = A(i, j)
  for (int c = c0 + warp; c < c1; c += nw) {
    double *x = X + (int64_t)c * m;
    double w = lane == 0 ? x[j] : 0.0;
    for (int64_t i = j + 1 + lane; i < m; i += 32) w += v[i] * x[i];
    for (int o = 16; o; o >>= 1) w += __shfl_xor_sync(0xffffffffu, w, o);
    w *= tau;
    if (lane == 0) x[j] -= w;
    for (int64_t i = j + 1 + lane; i < m; i += 32) x[i] -= w * v[i];
  }
}

__global__ void __launch_bounds__(512) qr_householder_kernel(const QrClass *cls, double *scr) {
  const QrClass C = cls[blockIdx.x];
  double *A = scr + C.a, *Q = scr + C.q, *tau = scr + C.t;
  const int m = C.m, n = C.n, k = m < n ? m : n;
  __shared__ double red[32];
  __shared__ double sh_tau, sh_scale;
  for (int j = 0; j < k; j++) {
    double *a = A + (int64_t)j * m;
    double part = 0;
    for (int64_t i = j + 1 + threadIdx.x; i < m; i += blockDim.x) part += a[i] * a[i];
    const double below = qr_block_sum(part, red);
    if (threadIdx.x == 0) {
      const double alpha = a[j], nrm = sqrt(alpha * alpha + below);
      if (below == 0.0) {
        sh_tau = 0.0;  // already zero below the diagonal: H_j = I
        sh_scale = 0.0;
      } else {
        const double beta = alpha >= 0 ? -nrm : nrm;
        sh_tau = (beta - alpha) / beta;
        sh_scale = 1.0 / (alpha - beta);
        a[j] = beta;
      }
      tau[j] = sh_tau;
    }
    __syncthreads();
    const double t = sh_tau, sc = sh_scale;
    if (t != 0.0)
      for (int64_t i = j + 1 + threadIdx.x; i < m; i += blockDim.x) a[i] *= sc;
    __syncthreads();
    if (t != 0.0) qr_apply(A, m, j, t, A, j + 1, n);
    __syncthreads();
  }
  // Q = H_0 ... H_{k-1} I(:, 0:k)
  for (int64_t e = threadIdx.x; e < (int64_t)m * k; e += blockDim.x)
    Q[e] = (e % m) == (e / m) ? 1.0 : 0.0;
  __syncthreads();
  for (int j = k - 1; j >= 0; j--) {
    const double t = tau[j];
    if (t != 0.0) qr_apply(A, m, j, t, Q, j, k);
    __syncthreads();
  }
  // non-negative diagonal of R: flip row i of R and column i of Q together
  for (int i = threadIdx.x; i < k; i += blockDim.x) tau[i] = A[(int64_t)i * m + i] < 0 ? -1.0 : 1.0;
  __syncthreads();
  for (int64_t e = threadIdx.x; e < (int64_t)m * k; e += blockDim.x) Q[e] *= tau[e / m];
  for (int64_t e = threadIdx.x; e < (int64_t)m * n; e += blockDim.x) {
    const int64_t i = e % m, c = e / m;
    if (i < k && i <= c) A[e] *= tau[i];
  }
}

// Output scatter of the QR factors: kind 0, a Q block (rows of X x the
// class's k), element (r, j) = Q(off + r, j); kind 1, an R block (k x columns
// of Y), element (i, c) = R(i, off + c), zero below the diagonal.
struct QrOut {
  int64_t dst, src;  // offset in the output's data; class Q or A in scratch
  int32_t m, k;      // class rows, bond size
  int32_t kind, off, len, pad;
};

__global__ void qr_scatter_kernel(const QrOut *ob, const int64_t *ostart, int64_t nob, int64_t ne,
                                  const double *scr, double *Qt, double *Rt) {
  const int64_t g = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (g >= ne) return;
  int64_t lo = 0, hi = nob - 1;
  while (lo < hi) {
    const int64_t mid = (lo + hi + 1) >> 1;
    if (ostart[mid] <= g) lo = mid; else hi = mid - 1;
  }
  const QrOut o = ob[lo];
  const int64_t e = g - ostart[lo];
  if (o.kind == 0) {
    const int64_t r = e % o.len, j = e / o.len;
    Qt[o.dst + e] = scr[o.src + (o.off + r) + j * (int64_t)o.m];
  } else {
    const int64_t i = e % o.k, c = o.off + e / o.k;
    Rt[o.dst + e] = i <= c ? scr[o.src + i + c * (int64_t)o.m] : 0.0;
  }
}

static int64_t box_size(const std::vector<int64_t> &box) {
  int64_t m = 1;
  for (size_t k = 0; k < box.size(); k += 2) m *= box[k + 1] - box[k] + 1;
  return m;
}

// The row-leg boxes X and column-leg boxes Y of a tensor and the classes they
// form (connected through blocks; the tensor is block diagonal over them):
// each class is one dense matrix, its X stacked as rows and its Y as columns
// in id order.
struct BoxClasses {
  std::vector<int32_t> rl, cl;                     // row legs, column legs
  std::vector<std::vector<int64_t>> xbox, ybox;    // (begin, end) per leg
  std::vector<int64_t> bx, by;                     // per block: its X and Y
  std::vector<int64_t> xoff, yoff, xc, yc;         // per X / Y: offset in, and id of, its class
  std::vector<std::vector<int64_t>> cx, cy;        // per class: its X and Y
  std::vector<int64_t> M, N;                       // per class: rows and columns
};

static tq_status box_classes(const tq_bs *T, int32_t n_row_legs, const int64_t *row_legs,
                             cudaStream_t s, BoxClasses &K) {
  const int32_t r = T->rank;
  std::vector<bool> used(r, false);
  for (int32_t q = 0; q < n_row_legs; q++) {
    if (row_legs[q] < 0 || row_legs[q] >= r || used[row_legs[q]])
      return fail(TQ_ERR_INVALID, "row legs out of range or repeated");
    used[row_legs[q]] = true;
    K.rl.push_back((int32_t)row_legs[q]);
  }
  for (int32_t l = 0; l < r; l++)
    if (!used[l]) K.cl.push_back(l);
  tq_bs *tm = const_cast<tq_bs *>(T);
  TQ_CHECK(sync_host_meta(tm, s));
  TQ_CHECK(sync_device_meta(tm, s));
  const int64_t nb = T->nb;
  // row / column boxes -> ids; intervals per leg must be equal or disjoint
  for (int32_t l = 0; l < r; l++) {
    std::vector<std::pair<int64_t, int64_t>> iv;
    for (int64_t b = 0; b < nb; b++) iv.push_back({T->h_begin[b * r + l], T->h_end[b * r + l]});
    std::sort(iv.begin(), iv.end());
    for (size_t k = 1; k < iv.size(); k++)
      if (iv[k] != iv[k - 1] && iv[k].first <= iv[k - 1].second)
        return fail(TQ_ERR_UNSUPPORTED, "the factorisations need sector boxes: intervals of a "
                                        "leg must be equal or disjoint");
  }
  std::map<std::vector<int64_t>, int64_t> xid, yid;
  K.bx.resize(nb);
  K.by.resize(nb);
  for (int64_t b = 0; b < nb; b++) {
    std::vector<int64_t> kx, ky;
    for (int32_t l : K.rl) kx.push_back(T->h_begin[b * r + l]), kx.push_back(T->h_end[b * r + l]);
    for (int32_t l : K.cl) ky.push_back(T->h_begin[b * r + l]), ky.push_back(T->h_end[b * r + l]);
    auto fx = xid.emplace(kx, (int64_t)K.xbox.size());
    if (fx.second) K.xbox.push_back(kx);
    auto fy = yid.emplace(ky, (int64_t)K.ybox.size());
    if (fy.second) K.ybox.push_back(ky);
    K.bx[b] = fx.first->second;
    K.by[b] = fy.first->second;
  }
  const int64_t nx = (int64_t)K.xbox.size(), ny = (int64_t)K.ybox.size();
  // classes: connected components of X and Y through blocks (union-find)
  std::vector<int64_t> par(nx + ny);
  std::iota(par.begin(), par.end(), 0);
  auto find = [&](int64_t a) {
    while (par[a] != a) a = par[a] = par[par[a]];
    return a;
  };
  for (int64_t b = 0; b < nb; b++) {
    const int64_t a = find(K.bx[b]), c = find(nx + K.by[b]);
    if (a != c) par[std::max(a, c)] = std::min(a, c);
  }
  std::map<int64_t, int64_t> cid;
  K.xoff.assign(nx, 0);
  K.yoff.assign(ny, 0);
  K.xc.assign(nx, -1);
  K.yc.assign(ny, -1);
  for (int64_t x = 0; x < nx; x++) {
    auto f = cid.emplace(find(x), (int64_t)K.cx.size());
    if (f.second) K.cx.emplace_back(), K.cy.emplace_back(), K.M.push_back(0), K.N.push_back(0);
    const int64_t c = f.first->second;
    K.xc[x] = c;
    K.xoff[x] = K.M[c];
    K.M[c] += box_size(K.xbox[x]);
    K.cx[c].push_back(x);
  }
  for (int64_t y = 0; y < ny; y++) {
    const int64_t c = cid.at(find(nx + y));
    K.yc[y] = c;
    K.yoff[y] = K.N[c];
    K.N[c] += box_size(K.ybox[y]);
    K.cy[c].push_back(y);
  }
  return TQ_OK;
}
}  // namespace tq

using namespace tq;

extern "C" tq_status tq_bs_svd(const tq_bs *T, int32_t n_row_legs, const int64_t *row_legs,
                               int64_t max_keep, double cutoff, tq_stream stream, tq_bs **U,
                               tq_bs **S, tq_bs **V) {
  if (!T || !U || !S || !V || (n_row_legs > 0 && !row_legs))
    return fail(TQ_ERR_INVALID, "NULL argument");
  if (T->dtype != TQ_F64) return fail(TQ_ERR_UNSUPPORTED, "the SVD takes float64 tensors");
  const int32_t r = T->rank;
  if (n_row_legs < 1 || n_row_legs >= r)
    return fail(TQ_ERR_INVALID, "need at least one row leg and one column leg");
  if (r + 1 > TQ_MAXR) return fail(TQ_ERR_UNSUPPORTED, "rank above 11");
  if (!(cutoff >= 0.0)) return fail(TQ_ERR_INVALID, "cutoff must be non-negative");
  cudaStream_t s = (cudaStream_t)stream;
  BoxClasses K;
  TQ_CHECK(box_classes(T, n_row_legs, row_legs, s, K));
  const std::vector<int32_t> &rl = K.rl, &cl = K.cl;
  const std::vector<std::vector<int64_t>> &xbox = K.xbox, &ybox = K.ybox, &cx = K.cx, &cy = K.cy;
  const std::vector<int64_t> &bx = K.bx, &by = K.by, &xoff = K.xoff, &yoff = K.yoff, &xc = K.xc;
  const std::vector<int64_t> &M = K.M, &N = K.N;
  const int64_t nb = T->nb;
  auto size_of = [](const std::vector<int64_t> &box) { return box_size(box); };
  const int64_t ncls = (int64_t)cx.size();
  // class scratch: matrix (oriented m >= n) then its n x n right factor
  std::vector<SvdClass> cls(ncls);
  std::vector<int64_t> sig_off(ncls + 1, 0);
  int64_t scr = 0;
  for (int64_t c = 0; c < ncls; c++) {
    const bool tr = M[c] < N[c];
    const int64_t m = tr ? N[c] : M[c], n = tr ? M[c] : N[c];
    if (m > 0x7fffffff) return fail(TQ_ERR_UNSUPPORTED, "a class above 2^31 rows");
    cls[c] = SvdClass{scr, scr + m * n, (int32_t)m, (int32_t)n, 0, 0};
    scr += m * n + n * n;
    sig_off[c + 1] = sig_off[c] + n;
  }
  std::vector<SvdBlock> sb(nb);
  std::vector<int64_t> estart(nb);
  int64_t ne = 0;
  for (int64_t b = 0; b < nb; b++) {
    const int64_t c = xc[bx[b]];
    const bool tr = M[c] < N[c];
    sb[b] = SvdBlock{cls[c].a, xoff[bx[b]], yoff[by[b]], cls[c].m, tr ? 1 : 0, 0};
    estart[b] = ne;
    int64_t e = 1;
    for (int32_t l = 0; l < r; l++) e *= T->h_end[b * r + l] - T->h_begin[b * r + l] + 1;
    ne += e;
  }
  DevArray<double> dscr, dsig;
  DevArray<SvdBlock> dsb;
  DevArray<SvdClass> dcls;
  DevArray<int64_t> dest, dsoff;
  DevArray<int32_t> dlegs, dinfo;
  TQ_CHECK(dscr.alloc(std::max<int64_t>(scr, 1), s));
  TQ_CHECK(dsig.alloc(std::max<int64_t>(sig_off[ncls], 1), s));
  TQ_CHECK(dsb.alloc(std::max<int64_t>(nb, 1), s));
  TQ_CHECK(dcls.alloc(std::max<int64_t>(ncls, 1), s));
  TQ_CHECK(dest.alloc(std::max<int64_t>(nb, 1), s));
  TQ_CHECK(dsoff.alloc(ncls + 1, s));
  TQ_CHECK(dlegs.alloc(r, s));
  TQ_CHECK(dinfo.alloc(1, s));
  std::vector<int32_t> legs(rl);
  legs.insert(legs.end(), cl.begin(), cl.end());
  TQ_CUDA(cudaMemsetAsync(dscr.p, 0, std::max<int64_t>(scr, 1) * 8, s));
  TQ_CUDA(cudaMemsetAsync(dinfo.p, 0, 4, s));
  if (nb) {
    TQ_CUDA(cudaMemcpyAsync(dsb.p, sb.data(), nb * sizeof(SvdBlock), cudaMemcpyHostToDevice, s));
    TQ_CUDA(cudaMemcpyAsync(dest.p, estart.data(), nb * 8, cudaMemcpyHostToDevice, s));
  }
  if (ncls)
    TQ_CUDA(cudaMemcpyAsync(dcls.p, cls.data(), ncls * sizeof(SvdClass), cudaMemcpyHostToDevice, s));
  TQ_CUDA(cudaMemcpyAsync(dsoff.p, sig_off.data(), (ncls + 1) * 8, cudaMemcpyHostToDevice, s));
  TQ_CUDA(cudaMemcpyAsync(dlegs.p, legs.data(), r * 4, cudaMemcpyHostToDevice, s));
  if (ne)
    count_launch(), svd_gather_kernel<<<blocks_of(ne), 256, 0, s>>>(
        T->view(), (int32_t)rl.size(), dlegs.p, (int32_t)cl.size(), dlegs.p + rl.size(), dsb.p,
        dest.p, ne, dscr.p);
  if (ncls)
    count_launch(), svd_jacobi_kernel<<<(unsigned)ncls, 512, 0, s>>>(dcls.p, dscr.p, dsig.p,
                                                                     dsoff.p, 40, dinfo.p);
  TQ_CUDA(cudaGetLastError());
  std::vector<double> sig(sig_off[ncls]);
  int32_t info = 0;
  if (!sig.empty())
    TQ_CUDA(cudaMemcpyAsync(sig.data(), dsig.p, sig.size() * 8, cudaMemcpyDeviceToHost, s));
  TQ_CUDA(cudaMemcpyAsync(&info, dinfo.p, 4, cudaMemcpyDeviceToHost, s));
  TQ_CUDA(cudaStreamSynchronize(s));
  if (info) return fail(TQ_ERR_CUDA, "the Jacobi SVD did not converge in 40 sweeps");
  // rank all values; keep the largest (at most max_keep, above cutoff * largest)
  std::vector<int32_t> perm(sig.size());
  std::vector<std::pair<double, int64_t>> all;
  double smax = 0;
  for (int64_t c = 0; c < ncls; c++) {
    int32_t *pc = perm.data() + sig_off[c];
    const int n = cls[c].n;
    std::iota(pc, pc + n, 0);
    std::stable_sort(pc, pc + n, [&](int32_t a, int32_t b) {
      return sig[sig_off[c] + a] > sig[sig_off[c] + b];
    });
    for (int k = 0; k < n; k++) {
      const double v = sig[sig_off[c] + pc[k]];
      all.push_back({v, c});
      smax = std::max(smax, v);
    }
  }
  std::stable_sort(all.begin(), all.end(),
                   [](const std::pair<double, int64_t> &a, const std::pair<double, int64_t> &b) {
                     return a.first > b.first;
                   });
  std::vector<int64_t> keep(ncls, 0);
  for (size_t k = 0; k < all.size(); k++) {
    if (max_keep > 0 && (int64_t)k >= max_keep) break;
    if (!(all[k].first > cutoff * smax) || all[k].first == 0.0) break;
    keep[all[k].second]++;
  }
  // the bond leg: one sector per class that keeps values, in class order
  std::vector<int64_t> bond_off(ncls, 0);
  int64_t bond = 0;
  for (int64_t c = 0; c < ncls; c++) bond_off[c] = bond, bond += keep[c];
  std::vector<int64_t> udim, vdim;
  for (int32_t l : rl) udim.push_back(T->dimension[l]);
  udim.push_back(std::max<int64_t>(bond, 1));
  vdim.push_back(std::max<int64_t>(bond, 1));
  for (int32_t l : cl) vdim.push_back(T->dimension[l]);
  std::vector<int64_t> ub, ue, vb, ve, sbeg, send;
  std::vector<SvdOut> ob;
  std::vector<int64_t> ostart;
  int64_t nu = 0, nv = 0, ns = 0, oe = 0;
  const int32_t ru = (int32_t)rl.size() + 1, rv = (int32_t)cl.size() + 1;
  for (int64_t c = 0; c < ncls; c++) {
    if (!keep[c]) continue;
    const bool tr = M[c] < N[c];
    for (int64_t x : cx[c]) {
      for (size_t k = 0; k < xbox[x].size(); k += 2) ub.push_back(xbox[x][k]), ue.push_back(xbox[x][k + 1]);
      ub.push_back(bond_off[c]);
      ue.push_back(bond_off[c] + keep[c] - 1);
      const int64_t len = size_of(xbox[x]);
      ob.push_back(SvdOut{nu, cls[c].a, cls[c].v, sig_off[c], sig_off[c], cls[c].m, cls[c].n, 0,
                          tr ? 1 : 0, (int32_t)xoff[x], (int32_t)len, (int32_t)keep[c], 0});
      ostart.push_back(oe);
      oe += len * keep[c];
      nu += len * keep[c];
    }
  }
  const int64_t n_ublk = (int64_t)ob.size();
  for (int64_t c = 0; c < ncls; c++) {
    if (!keep[c]) continue;
    const bool tr = M[c] < N[c];
    for (int64_t y : cy[c]) {
      vb.push_back(bond_off[c]);
      ve.push_back(bond_off[c] + keep[c] - 1);
      for (size_t k = 0; k < ybox[y].size(); k += 2) vb.push_back(ybox[y][k]), ve.push_back(ybox[y][k + 1]);
      const int64_t len = size_of(ybox[y]);
      ob.push_back(SvdOut{nv, cls[c].a, cls[c].v, sig_off[c], sig_off[c], cls[c].m, cls[c].n, 1,
                          tr ? 1 : 0, (int32_t)yoff[y], (int32_t)len, (int32_t)keep[c], 0});
      ostart.push_back(oe);
      oe += len * keep[c];
      nv += len * keep[c];
    }
  }
  const int64_t n_vblk = (int64_t)ob.size() - n_ublk;
  for (int64_t c = 0; c < ncls; c++) {
    if (!keep[c]) continue;
    sbeg.push_back(bond_off[c]);
    send.push_back(bond_off[c] + keep[c] - 1);
    ob.push_back(SvdOut{ns, 0, 0, sig_off[c], sig_off[c], cls[c].m, cls[c].n, 2, 0, 0,
                        (int32_t)keep[c], (int32_t)keep[c], 0});
    ostart.push_back(oe);
    oe += keep[c];
    ns += keep[c];
  }
  tq_bs *Ut = nullptr, *St = nullptr, *Vt = nullptr;
  int64_t sdim = std::max<int64_t>(bond, 1);
  TQ_CHECK(tq_bs_create_zeros(TQ_F64, ru, udim.data(), n_ublk, ub.data(), ue.data(), nullptr,
                              stream, &Ut));
  std::unique_ptr<tq_bs, tq_status (*)(tq_bs *)> gu(Ut, tq_bs_destroy);
  TQ_CHECK(tq_bs_create_zeros(TQ_F64, rv, vdim.data(), n_vblk, vb.data(), ve.data(), nullptr,
                              stream, &Vt));
  std::unique_ptr<tq_bs, tq_status (*)(tq_bs *)> gv(Vt, tq_bs_destroy);
  TQ_CHECK(tq_bs_create_zeros(TQ_F64, 1, &sdim, (int64_t)sbeg.size(), sbeg.data(), send.data(),
                              nullptr, stream, &St));
  std::unique_ptr<tq_bs, tq_status (*)(tq_bs *)> gs(St, tq_bs_destroy);
  if (oe) {
    DevArray<SvdOut> dob;
    DevArray<int64_t> dos;
    DevArray<int32_t> dperm;
    TQ_CHECK(dob.alloc(ob.size(), s));
    TQ_CHECK(dos.alloc(ostart.size(), s));
    TQ_CHECK(dperm.alloc(std::max<size_t>(perm.size(), 1), s));
    TQ_CUDA(cudaMemcpyAsync(dob.p, ob.data(), ob.size() * sizeof(SvdOut), cudaMemcpyHostToDevice, s));
    TQ_CUDA(cudaMemcpyAsync(dos.p, ostart.data(), ostart.size() * 8, cudaMemcpyHostToDevice, s));
    TQ_CUDA(cudaMemcpyAsync(dperm.p, perm.data(), perm.size() * 4, cudaMemcpyHostToDevice, s));
    count_launch(), svd_scatter_kernel<<<blocks_of(oe), 256, 0, s>>>(
        dob.p, dos.p, (int64_t)ob.size(), oe, dscr.p, dsig.p, dperm.p, (double *)Ut->data,
        (double *)St->data, (double *)Vt->data);
    TQ_CUDA(cudaGetLastError());
    TQ_CUDA(cudaStreamSynchronize(s));  // host staging dies here
  }
  *U = gu.release();
  *S = gs.release();
  *V = gv.release();
  return TQ_OK;
}

extern "C" tq_status tq_bs_qr(const tq_bs *T, int32_t n_row_legs, const int64_t *row_legs,
                              tq_stream stream, tq_bs **Qo, tq_bs **Ro) {
  if (!T || !Qo || !Ro || (n_row_legs > 0 && !row_legs))
    return fail(TQ_ERR_INVALID, "NULL argument");
  if (T->dtype != TQ_F64) return fail(TQ_ERR_UNSUPPORTED, "the QR takes float64 tensors");
  const int32_t r = T->rank;
  if (n_row_legs < 1 || n_row_legs >= r)
    return fail(TQ_ERR_INVALID, "need at least one row leg and one column leg");
  if (r + 1 > TQ_MAXR) return fail(TQ_ERR_UNSUPPORTED, "rank above 11");
  cudaStream_t s = (cudaStream_t)stream;
  BoxClasses K;
  TQ_CHECK(box_classes(T, n_row_legs, row_legs, s, K));
  const int64_t nb = T->nb, ncls = (int64_t)K.cx.size();
  std::vector<QrClass> cls(ncls);
  std::vector<int64_t> kc(ncls), bond_off(ncls);
  int64_t scr = 0, bond = 0;
  for (int64_t c = 0; c < ncls; c++) {
    const int64_t m = K.M[c], n = K.N[c], k = std::min(m, n);
    if (m > 0x7fffffff || n > 0x7fffffff) return fail(TQ_ERR_UNSUPPORTED, "a class above 2^31 rows");
    cls[c] = QrClass{scr, scr + m * n, scr + m * n + m * k, (int32_t)m, (int32_t)n};
    scr += m * n + m * k + k;
    kc[c] = k;
    bond_off[c] = bond;
    bond += k;
  }
  std::vector<SvdBlock> sb(nb);
  std::vector<int64_t> estart(nb);
  int64_t ne = 0;
  for (int64_t b = 0; b < nb; b++) {
    const int64_t c = K.xc[K.bx[b]];
    sb[b] = SvdBlock{cls[c].a, K.xoff[K.bx[b]], K.yoff[K.by[b]], cls[c].m, 0, 0};
    estart[b] = ne;
    int64_t e = 1;
    for (int32_t l = 0; l < r; l++) e *= T->h_end[b * r + l] - T->h_begin[b * r + l] + 1;
    ne += e;
  }
  DevArray<double> dscr;
  DevArray<SvdBlock> dsb;
  DevArray<QrClass> dcls;
  DevArray<int64_t> dest;
  DevArray<int32_t> dlegs;
  TQ_CHECK(dscr.alloc(std::max<int64_t>(scr, 1), s));
  TQ_CHECK(dsb.alloc(std::max<int64_t>(nb, 1), s));
  TQ_CHECK(dcls.alloc(std::max<int64_t>(ncls, 1), s));
  TQ_CHECK(dest.alloc(std::max<int64_t>(nb, 1), s));
  TQ_CHECK(dlegs.alloc(r, s));
  std::vector<int32_t> legs(K.rl);
  legs.insert(legs.end(), K.cl.begin(), K.cl.end());
  TQ_CUDA(cudaMemsetAsync(dscr.p, 0, std::max<int64_t>(scr, 1) * 8, s));
  if (nb) {
    TQ_CUDA(cudaMemcpyAsync(dsb.p, sb.data(), nb * sizeof(SvdBlock), cudaMemcpyHostToDevice, s));
    TQ_CUDA(cudaMemcpyAsync(dest.p, estart.data(), nb * 8, cudaMemcpyHostToDevice, s));
  }
  if (ncls)
    TQ_CUDA(cudaMemcpyAsync(dcls.p, cls.data(), ncls * sizeof(QrClass), cudaMemcpyHostToDevice, s));
  TQ_CUDA(cudaMemcpyAsync(dlegs.p, legs.data(), r * 4, cudaMemcpyHostToDevice, s));
  if (ne)
    count_launch(), svd_gather_kernel<<<blocks_of(ne), 256, 0, s>>>(
        T->view(), (int32_t)K.rl.size(), dlegs.p, (int32_t)K.cl.size(), dlegs.p + K.rl.size(),
        dsb.p, dest.p, ne, dscr.p);
  if (ncls) count_launch(), qr_householder_kernel<<<(unsigned)ncls, 512, 0, s>>>(dcls.p, dscr.p);
  TQ_CUDA(cudaGetLastError());
  // the factors over a new bond leg, one sector of min(M, N) per class
  std::vector<int64_t> qdim, rdim;
  for (int32_t l : K.rl) qdim.push_back(T->dimension[l]);
  qdim.push_back(std::max<int64_t>(bond, 1));
  rdim.push_back(std::max<int64_t>(bond, 1));
  for (int32_t l : K.cl) rdim.push_back(T->dimension[l]);
  std::vector<int64_t> qb, qe, rb, re, ostart;
  std::vector<QrOut> ob;
  int64_t nq = 0, nr = 0, oe = 0;
  for (int64_t c = 0; c < ncls; c++) {
    if (!kc[c]) continue;
    for (int64_t x : K.cx[c]) {
      for (size_t q = 0; q < K.xbox[x].size(); q += 2)
        qb.push_back(K.xbox[x][q]), qe.push_back(K.xbox[x][q + 1]);
      qb.push_back(bond_off[c]);
      qe.push_back(bond_off[c] + kc[c] - 1);
      const int64_t len = box_size(K.xbox[x]);
      ob.push_back(QrOut{nq, cls[c].q, cls[c].m, (int32_t)kc[c], 0, (int32_t)K.xoff[x],
                         (int32_t)len, 0});
      ostart.push_back(oe);
      oe += len * kc[c];
      nq += len * kc[c];
    }
  }
  const int64_t n_qblk = (int64_t)ob.size();
  for (int64_t c = 0; c < ncls; c++) {
    if (!kc[c]) continue;
    for (int64_t y : K.cy[c]) {
      rb.push_back(bond_off[c]);
      re.push_back(bond_off[c] + kc[c] - 1);
      for (size_t q = 0; q < K.ybox[y].size(); q += 2)
        rb.push_back(K.ybox[y][q]), re.push_back(K.ybox[y][q + 1]);
      const int64_t len = box_size(K.ybox[y]);
      ob.push_back(QrOut{nr, cls[c].a, cls[c].m, (int32_t)kc[c], 1, (int32_t)K.yoff[y],
                         (int32_t)len, 0});
      ostart.push_back(oe);
      oe += len * kc[c];
      nr += len * kc[c];
    }
  }
  const int64_t n_rblk = (int64_t)ob.size() - n_qblk;
  tq_bs *Qt = nullptr, *Rt = nullptr;
  TQ_CHECK(tq_bs_create_zeros(TQ_F64, (int32_t)K.rl.size() + 1, qdim.data(), n_qblk, qb.data(),
                              qe.data(), nullptr, stream, &Qt));
  std::unique_ptr<tq_bs, tq_status (*)(tq_bs *)> gq(Qt, tq_bs_destroy);
  TQ_CHECK(tq_bs_create_zeros(TQ_F64, (int32_t)K.cl.size() + 1, rdim.data(), n_rblk, rb.data(),
                              re.data(), nullptr, stream, &Rt));
  std::unique_ptr<tq_bs, tq_status (*)(tq_bs *)> gr(Rt, tq_bs_destroy);
  if (oe) {
    DevArray<QrOut> dob;
    DevArray<int64_t> dos;
    TQ_CHECK(dob.alloc(ob.size(), s));
    TQ_CHECK(dos.alloc(ostart.size(), s));
    TQ_CUDA(cudaMemcpyAsync(dob.p, ob.data(), ob.size() * sizeof(QrOut), cudaMemcpyHostToDevice, s));
    TQ_CUDA(cudaMemcpyAsync(dos.p, ostart.data(), ostart.size() * 8, cudaMemcpyHostToDevice, s));
    count_launch(), qr_scatter_kernel<<<blocks_of(oe), 256, 0, s>>>(
        dob.p, dos.p, (int64_t)ob.size(), oe, dscr.p, (double *)Qt->data, (double *)Rt->data);
    TQ_CUDA(cudaGetLastError());
  }
  TQ_CUDA(cudaStreamSynchronize(s));  // host staging dies here
  *Qo = gq.release();
  *Ro = gr.release();
  return TQ_OK;
}
