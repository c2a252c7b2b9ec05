// Element-sparse contraction by sort-join (the GPU sparse path of the
// reference, src/gpu/sparse.cuh:270-375, without its all-pairs step).
//
// The reference forms the outer product of all nonzeros of A with all of B
// (one rank-1 GEMM, nnz_A x nnz_B values, src/gpu/sparse.cuh:320-350), gives
// every product an output index (or a sentinel for non-matching pairs), sorts
// them and reduces by key.  Here both operands are sorted by their contracted
// index and only the matching runs are multiplied: O(nnz log nnz + products)
// work and memory instead of O(nnz_A nnz_B).
//
// An element-sparse tensor is a block-sparse tensor whose blocks each hold one
// element (the SparseTensor classes build them so).  Steps: per element, its
// contracted key (linear index over the contracted legs, pair order, first
// fastest) and free key; stable radix sorts by contracted key; per A element
// the run of B elements with its key (binary search); products emitted with
// their output index (A free legs then B free legs, column-major); a stable
// sort by output index and a fixed-order sum per output element; one
// one-element block per distinct output element, in output-index order.
#include <cuda_fp16.h>

#include <vector>

#include "index.cuh"
#include "tq_internal.h"

namespace tq {

static inline unsigned blocks_for(int64_t n) { return (unsigned)((n + 255) / 256); }

struct KeyTables {
  int32_t nc, nf;
  int32_t con[TQ_MAXR], fre[TQ_MAXR];
  int64_t ctab[TQ_MAXR], ftab[TQ_MAXR];
};

__global__ void elem_keys_kernel(DevBS T, KeyTables K, int64_t *ckey, int64_t *fkey,
                                 int64_t *perm, int32_t *bad) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= T.nb) return;
  const int64_t *b = T.begin + i * T.rank, *e = T.end + i * T.rank;
  int64_t c = 0, f = 0;
  for (int l = 0; l < T.rank; l++)
    if (b[l] != e[l]) atomicOr(bad, 1);  // not a one-element block
  for (int q = 0; q < K.nc; q++) c += b[K.con[q]] * K.ctab[q];
  for (int q = 0; q < K.nf; q++) f += b[K.fre[q]] * K.ftab[q];
  ckey[i] = c;
  fkey[i] = f;
  perm[i] = i;
}

// lower_bound of x in sorted k[0..n)
__device__ __forceinline__ int64_t lower(const int64_t *k, int64_t n, int64_t x) {
  int64_t lo = 0, hi = n;
  while (lo < hi) {
    const int64_t mid = (lo + hi) >> 1;
    if (k[mid] < x) lo = mid + 1; else hi = mid;
  }
  return lo;
}

// per sorted A element: first matching B position and run length
__global__ void run_kernel(const int64_t *ka, int64_t na, const int64_t *kb, int64_t nb,
                           int64_t *first, int64_t *count) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= na) return;
  const int64_t x = ka[i];
  const int64_t lo = lower(kb, nb, x), hi = lower(kb, nb, x + 1);
  first[i] = lo;
  count[i] = hi - lo;
}

template <typename T>
__device__ __forceinline__ double as_double(const T *d, int64_t i) { return (double)d[i]; }
template <>
__device__ __forceinline__ double as_double<__half>(const __half *d, int64_t i) {
  return (double)__half2float(d[i]);
}

// products of sorted A element i with its B run: output index and value (FP64
// for every element type, rounded once when the sum is stored)
template <typename T>
__global__ void emit_kernel(const int64_t *pa, const int64_t *pb, const int64_t *fa,
                            const int64_t *fb, const int64_t *first, const int64_t *count,
                            const int64_t *start, int64_t na, int64_t MA, const T *ad,
                            const int64_t *aoff, const T *bd, const int64_t *boff,
                            int64_t *okey, int64_t *oidx, double *oval) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= na) return;
  const int64_t a = pa[i];
  const double av = as_double(ad, aoff[a]);
  const int64_t fA = fa[a];
  for (int64_t q = 0; q < count[i]; q++) {
    const int64_t j = pb[first[i] + q];
    const int64_t o = start[i] + q;
    okey[o] = fA + MA * fb[j];
    oidx[o] = o;
    oval[o] = av * as_double(bd, boff[j]);
  }
}

// one thread per output element: its products summed in FP64 in emission
// order, rounded to the element type once
__device__ __forceinline__ void store_elem(double *o, double v) { *o = v; }
__device__ __forceinline__ void store_elem(float *o, double v) { *o = (float)v; }
__device__ __forceinline__ void store_elem(__half *o, double v) { *o = __double2half(v); }

template <typename T>
__global__ void reduce_kernel(const int64_t *okey, const int64_t *oidx, const double *oval,
                              const int64_t *seg, int64_t nu, int32_t rank, const int64_t *ndim,
                              int64_t *begin, int64_t *end, int64_t *strides, int64_t *offsets,
                              T *out) {
  const int64_t u = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (u >= nu) return;
  double acc = 0.0;
  for (int64_t s = seg[u]; s < seg[u + 1]; s++) acc += oval[oidx[s]];
  int64_t x = okey[seg[u]];
  for (int l = 0; l < rank; l++) {
    const int64_t c = x % ndim[l];
    x /= ndim[l];
    begin[u * rank + l] = c;
    end[u * rank + l] = c;
    strides[u * rank + l] = 1;
  }
  offsets[u] = u;
  store_elem(out + u, acc);
}

__global__ void head_kernel(const int64_t *key, int64_t n, int64_t *flag) {
  const int64_t s = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (s < n) flag[s] = (s == 0 || key[s] != key[s - 1]) ? 1 : 0;
}

__global__ void seg_kernel(const int64_t *flag, const int64_t *sid, int64_t n, int64_t nu,
                           int64_t *seg) {
  const int64_t s = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (s < n && flag[s]) seg[sid[s]] = s;
  if (s == 0) seg[nu] = n;
}

static int key_bits(int64_t K) {
  int b = 0;
  while (b < 63 && (int64_t(1) << b) < K) b++;
  return b;
}

static tq_status keys_for(const tq_bs *T, const LegSpec &L, bool is_a, const int64_t *dim,
                          KeyTables &K, int64_t *range_c, int64_t *range_f) {
  K.nc = L.nc;
  K.nf = is_a ? L.nfa : L.nfb;
  int64_t r = 1;
  for (int q = 0; q < L.nc; q++) {
    K.con[q] = is_a ? L.al[q] : L.bl[q];
    K.ctab[q] = r;
    const int64_t d = T->dimension[K.con[q]];
    if (d > 0 && r > (int64_t(1) << 62) / d) return fail(TQ_ERR_UNSUPPORTED, "index range above 2^62");
    r *= d;
  }
  *range_c = r;
  r = 1;
  for (int q = 0; q < K.nf; q++) {
    K.fre[q] = is_a ? L.fa[q] : L.fb[q];
    K.ftab[q] = r;
    const int64_t d = T->dimension[K.fre[q]];
    if (d > 0 && r > (int64_t(1) << 62) / d) return fail(TQ_ERR_UNSUPPORTED, "index range above 2^62");
    r *= d;
  }
  *range_f = r;
  (void)dim;
  return TQ_OK;
}

tq_status validate_legs(const tq_bs *A, const tq_bs *B, int32_t n_legs, const int64_t *a_legs,
                        const int64_t *b_legs, LegSpec &L);

}  // namespace tq

using namespace tq;

extern "C" tq_status tq_bs_contract_elements(const tq_bs *A, const tq_bs *B, int32_t n_legs,
                                             const int64_t *a_legs, const int64_t *b_legs,
                                             tq_stream stream, tq_bs **out) {
  if (!out) return fail(TQ_ERR_INVALID, "out is NULL");
  LegSpec L;
  TQ_CHECK(validate_legs(A, B, n_legs, a_legs, b_legs, L));
  const int32_t rc = L.nfa + L.nfb;
  if (rc == 0) return fail(TQ_ERR_UNSUPPORTED, "element contraction to a scalar: use tq_bs_contract");
  cudaStream_t s = (cudaStream_t)stream;
  TQ_CHECK(sync_device_meta(const_cast<tq_bs *>(A), s));
  TQ_CHECK(sync_device_meta(const_cast<tq_bs *>(B), s));
  std::vector<int64_t> ndim;
  for (int q = 0; q < L.nfa; q++) ndim.push_back(A->dimension[L.fa[q]]);
  for (int q = 0; q < L.nfb; q++) ndim.push_back(B->dimension[L.fb[q]]);
  KeyTables KA_, KB_;
  int64_t rca, rfa, rcb, rfb;
  TQ_CHECK(keys_for(A, L, true, ndim.data(), KA_, &rca, &rfa));
  TQ_CHECK(keys_for(B, L, false, ndim.data(), KB_, &rcb, &rfb));
  if (rfb > 0 && rfa > (int64_t(1) << 62) / rfb)
    return fail(TQ_ERR_UNSUPPORTED, "output index range above 2^62");
  const int64_t na = A->nb, nb = B->nb;
  DevArray<int64_t> cka, fka, pa, ckb, fkb, pb;
  DevArray<int32_t> bad;
  TQ_CHECK(cka.alloc(std::max<int64_t>(na, 1), s));
  TQ_CHECK(fka.alloc(std::max<int64_t>(na, 1), s));
  TQ_CHECK(pa.alloc(std::max<int64_t>(na, 1), s));
  TQ_CHECK(ckb.alloc(std::max<int64_t>(nb, 1), s));
  TQ_CHECK(fkb.alloc(std::max<int64_t>(nb, 1), s));
  TQ_CHECK(pb.alloc(std::max<int64_t>(nb, 1), s));
  TQ_CHECK(bad.alloc(1, s));
  TQ_CUDA(cudaMemsetAsync(bad.p, 0, 4, s));
  if (na) count_launch(), elem_keys_kernel<<<blocks_for(na), 256, 0, s>>>(A->view(), KA_, cka.p, fka.p, pa.p, bad.p);
  if (nb) count_launch(), elem_keys_kernel<<<blocks_for(nb), 256, 0, s>>>(B->view(), KB_, ckb.p, fkb.p, pb.p, bad.p);
  TQ_CUDA(cudaGetLastError());
  // stable sorts by contracted key (ties keep block order)
  if (na) TQ_CHECK(radix_sort_pairs(cka.p, pa.p, na, key_bits(rca), s));
  if (nb) TQ_CHECK(radix_sort_pairs(ckb.p, pb.p, nb, key_bits(rcb), s));
  DevArray<int64_t> first, cnt, start, tot;
  TQ_CHECK(first.alloc(std::max<int64_t>(na, 1), s));
  TQ_CHECK(cnt.alloc(std::max<int64_t>(na, 1), s));
  TQ_CHECK(start.alloc(std::max<int64_t>(na, 1), s));
  TQ_CHECK(tot.alloc(2, s));
  if (na) count_launch(), run_kernel<<<blocks_for(na), 256, 0, s>>>(cka.p, na, ckb.p, nb, first.p, cnt.p);
  TQ_CUDA(cudaGetLastError());
  TQ_CHECK(scan_exclusive(cnt.p, start.p, na, tot.p, s));
  int64_t np_ = 0;
  int32_t h_bad = 0;
  TQ_CUDA(cudaMemcpyAsync(&np_, tot.p, 8, cudaMemcpyDeviceToHost, s));
  TQ_CUDA(cudaMemcpyAsync(&h_bad, bad.p, 4, cudaMemcpyDeviceToHost, s));
  TQ_CUDA(cudaStreamSynchronize(s));
  if (h_bad) return fail(TQ_ERR_INVALID, "element contraction needs one-element blocks");
  if (na == 0 || nb == 0) np_ = 0;
  DevArray<int64_t> okey, oidx;
  DevArray<double> oval;
  TQ_CHECK(okey.alloc(std::max<int64_t>(np_, 1), s));
  TQ_CHECK(oidx.alloc(std::max<int64_t>(np_, 1), s));
  TQ_CHECK(oval.alloc(std::max<int64_t>(np_, 1), s));
  const DevBS av = A->view(), bv = B->view();
  if (np_) {
    const unsigned g = blocks_for(na);
    count_launch();
    if (A->dtype == TQ_F64)
      emit_kernel<double><<<g, 256, 0, s>>>(pa.p, pb.p, fka.p, fkb.p, first.p, cnt.p, start.p, na,
                                            rfa, (const double *)av.data, av.offsets,
                                            (const double *)bv.data, bv.offsets, okey.p, oidx.p,
                                            oval.p);
    else if (A->dtype == TQ_F32)
      emit_kernel<float><<<g, 256, 0, s>>>(pa.p, pb.p, fka.p, fkb.p, first.p, cnt.p, start.p, na,
                                           rfa, (const float *)av.data, av.offsets,
                                           (const float *)bv.data, bv.offsets, okey.p, oidx.p,
                                           oval.p);
    else
      emit_kernel<__half><<<g, 256, 0, s>>>(pa.p, pb.p, fka.p, fkb.p, first.p, cnt.p, start.p, na,
                                            rfa, (const __half *)av.data, av.offsets,
                                            (const __half *)bv.data, bv.offsets, okey.p, oidx.p,
                                            oval.p);
    TQ_CUDA(cudaGetLastError());
    TQ_CHECK(radix_sort_pairs(okey.p, oidx.p, np_, key_bits(rfa * rfb), s));
  }
  // distinct output elements
  DevArray<int64_t> flag, sid, seg;
  TQ_CHECK(flag.alloc(std::max<int64_t>(np_, 1), s));
  TQ_CHECK(sid.alloc(std::max<int64_t>(np_, 1), s));
  int64_t nu = 0;
  if (np_) {
    count_launch(), head_kernel<<<blocks_for(np_), 256, 0, s>>>(okey.p, np_, flag.p);
    TQ_CHECK(scan_exclusive(flag.p, sid.p, np_, tot.p + 1, s));
    TQ_CUDA(cudaMemcpyAsync(&nu, tot.p + 1, 8, cudaMemcpyDeviceToHost, s));
    TQ_CUDA(cudaStreamSynchronize(s));
  }
  TQ_CHECK(seg.alloc(nu + 1, s));
  if (np_) count_launch(), seg_kernel<<<blocks_for(np_), 256, 0, s>>>(flag.p, sid.p, np_, nu, seg.p);
  TQ_CUDA(cudaGetLastError());
  tq_bs *C = new_tensor(A->dtype, rc, ndim.data());
  std::unique_ptr<tq_bs, tq_status (*)(tq_bs *)> guard(C, tq_bs_destroy);
  C->nb = nu;
  TQ_CHECK(C->d_meta.alloc(3 * (size_t)nu * rc + nu, s));
  TQ_CHECK(alloc_data(C, nu, s));
  DevArray<int64_t> dd;
  TQ_CHECK(dd.alloc(rc, s));
  TQ_CUDA(cudaMemcpyAsync(dd.p, ndim.data(), rc * 8, cudaMemcpyHostToDevice, s));
  if (nu) {
    int64_t *cb = C->d_meta.p, *ce = cb + nu * rc, *cs = ce + nu * rc, *co = cs + nu * rc;
    const unsigned g = blocks_for(nu);
    count_launch();
    if (A->dtype == TQ_F64)
      reduce_kernel<double><<<g, 256, 0, s>>>(okey.p, oidx.p, oval.p, seg.p, nu, rc, dd.p,
                                                      cb, ce, cs, co, (double *)C->data);
    else if (A->dtype == TQ_F32)
      reduce_kernel<float><<<g, 256, 0, s>>>(okey.p, oidx.p, oval.p, seg.p, nu, rc, dd.p,
                                                    cb, ce, cs, co, (float *)C->data);
    else
      reduce_kernel<__half><<<g, 256, 0, s>>>(okey.p, oidx.p, oval.p, seg.p, nu, rc, dd.p,
                                                     cb, ce, cs, co, (__half *)C->data);
    TQ_CUDA(cudaGetLastError());
  }
  TQ_CUDA(cudaStreamSynchronize(s));  // ndim (host staging) dies here
  C->host_valid = false;
  C->dev_valid = true;
  *out = guard.release();
  return TQ_OK;
}
