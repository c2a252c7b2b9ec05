// Leg fusion by charge sectors: legs i and i+1 of a block-sparse tensor become
// one leg whose index space is the (sector_a, sector_b) pairs laid end to end
// in the caller's order (charge-sorted for symmetric tensors), each pair a
// contiguous range of size_a * size_b.
//
// A block that covers whole sectors on both legs keeps its data untouched: in
// column-major order its (x_a, x_b) elements already sit at x_a + size_a * x_b,
// which is the fused index inside the pair's range.  So fusion rewrites the
// boxes and strides (one thread per block) and copies the data buffer as is.
// The reference has no leg fusion; a PEPS double layer (D x D -> D^2) needs it.
#include <algorithm>
#include <cstring>
#include <vector>

#include "tq_internal.h"

namespace tq {

__device__ __forceinline__ int64_t sector_of(const int64_t *bounds, int64_t n, int64_t x) {
  // largest s with bounds[s] <= x (bounds[0] = 0, bounds[n] = dim)
  int64_t lo = 0, hi = n - 1;
  while (lo < hi) {
    const int64_t mid = (lo + hi + 1) >> 1;
    if (bounds[mid] <= x) lo = mid; else hi = mid - 1;
  }
  return lo;
}

__global__ void fuse_kernel(DevBS T, int32_t leg, const int64_t *ba, int64_t na,
                            const int64_t *bb, int64_t nb, const int64_t *off, int64_t *nbeg,
                            int64_t *nend, int64_t *nstr, int32_t *bad) {
  const int64_t b = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (b >= T.nb) return;
  const int32_t r = T.rank, nr = r - 1;
  const int64_t xa = T.begin[b * r + leg], ya = T.end[b * r + leg];
  const int64_t xb = T.begin[b * r + leg + 1], yb = T.end[b * r + leg + 1];
  const int64_t sa = sector_of(ba, na, xa), sb = sector_of(bb, nb, xb);
  const int64_t size_a = ba[sa + 1] - ba[sa], size_b = bb[sb + 1] - bb[sb];
  const int64_t st_a = T.strides[b * r + leg], st_b = T.strides[b * r + leg + 1];
  if (xa != ba[sa] || ya != ba[sa + 1] - 1 || xb != bb[sb] || yb != bb[sb + 1] - 1 ||
      st_b != st_a * size_a) {
    atomicOr(bad, 1);
    return;
  }
  const int64_t o = off[sa + na * sb];
  for (int32_t l = 0, q = 0; l < r; l++) {
    if (l == leg + 1) continue;
    if (l == leg) {
      nbeg[b * nr + q] = o;
      nend[b * nr + q] = o + size_a * size_b - 1;
      nstr[b * nr + q] = st_a;
    } else {
      nbeg[b * nr + q] = T.begin[b * r + l];
      nend[b * nr + q] = T.end[b * r + l];
      nstr[b * nr + q] = T.strides[b * r + l];
    }
    q++;
  }
}

// Inverse of fuse_kernel: a block whose box on the fused leg is exactly one
// sector pair's range becomes the pair's two sector boxes; strides st and
// st * size_a (its column-major data are already in that layout).  pstart /
// pidx: the pair ranges' starts, ascending, and their pair index a + na * b.
__global__ void split_kernel(DevBS T, int32_t leg, const int64_t *ba, int64_t na,
                             const int64_t *bb, const int64_t *pstart, const int64_t *pidx,
                             int64_t npairs, int64_t *nbeg, int64_t *nend, int64_t *nstr,
                             int32_t *bad) {
  const int64_t b = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (b >= T.nb) return;
  const int32_t r = T.rank, nr = r + 1;
  const int64_t x = T.begin[b * r + leg], y = T.end[b * r + leg];
  const int64_t k = sector_of(pstart, npairs, x);
  const int64_t pa = pidx[k] % na, pb = pidx[k] / na;
  const int64_t size_a = ba[pa + 1] - ba[pa], size_b = bb[pb + 1] - bb[pb];
  if (x != pstart[k] || y != x + size_a * size_b - 1) {
    atomicOr(bad, 1);
    return;
  }
  const int64_t st = T.strides[b * r + leg];
  for (int32_t l = 0, q = 0; l < r; l++, q++) {
    if (l == leg) {
      nbeg[b * nr + q] = ba[pa];
      nend[b * nr + q] = ba[pa + 1] - 1;
      nstr[b * nr + q] = st;
      q++;
      nbeg[b * nr + q] = bb[pb];
      nend[b * nr + q] = bb[pb + 1] - 1;
      nstr[b * nr + q] = st * size_a;
    } else {
      nbeg[b * nr + q] = T.begin[b * r + l];
      nend[b * nr + q] = T.end[b * r + l];
      nstr[b * nr + q] = T.strides[b * r + l];
    }
  }
}

// The pair ranges of a fusion tile [0, dim_a * dim_b) exactly (shared check).
static tq_status check_pairs(int64_t n_sec_a, const int64_t *bounds_a, int64_t n_sec_b,
                             const int64_t *bounds_b, const int64_t *pair_offset,
                             int64_t fused) {
  for (int64_t s = 0; s < n_sec_a; s++)
    if (bounds_a[s + 1] <= bounds_a[s]) return fail(TQ_ERR_INVALID, "sector bounds not increasing");
  for (int64_t s = 0; s < n_sec_b; s++)
    if (bounds_b[s + 1] <= bounds_b[s]) return fail(TQ_ERR_INVALID, "sector bounds not increasing");
  std::vector<std::pair<int64_t, int64_t>> rng;
  for (int64_t b = 0; b < n_sec_b; b++)
    for (int64_t a = 0; a < n_sec_a; a++)
      rng.push_back({pair_offset[a + n_sec_a * b],
                     (bounds_a[a + 1] - bounds_a[a]) * (bounds_b[b + 1] - bounds_b[b])});
  std::sort(rng.begin(), rng.end());
  int64_t run = 0;
  for (auto &x : rng) {
    if (x.first != run) return fail(TQ_ERR_INVALID, "pair offsets do not tile the fused leg");
    run += x.second;
  }
  if (run != fused) return fail(TQ_ERR_INVALID, "pair offsets do not tile the fused leg");
  return TQ_OK;
}

}  // namespace tq

using namespace tq;

extern "C" {

tq_status tq_bs_split_leg(const tq_bs *t, int32_t leg, int64_t n_sec_a, const int64_t *bounds_a,
                          int64_t n_sec_b, const int64_t *bounds_b, const int64_t *pair_offset,
                          tq_stream stream, tq_bs **out) {
  if (!t || !out || !bounds_a || !bounds_b || !pair_offset)
    return fail(TQ_ERR_INVALID, "NULL argument");
  if (leg < 0 || leg >= t->rank) return fail(TQ_ERR_INVALID, "leg to split out of range");
  if (t->rank + 1 > TQ_MAXR) return fail(TQ_ERR_UNSUPPORTED, "result rank above 12");
  if (n_sec_a <= 0 || n_sec_b <= 0) return fail(TQ_ERR_INVALID, "empty sector list");
  if (bounds_a[0] != 0 || bounds_b[0] != 0 ||
      bounds_a[n_sec_a] * bounds_b[n_sec_b] != t->dimension[leg])
    return fail(TQ_ERR_INVALID, "sector bounds do not span the leg to split");
  TQ_CHECK(check_pairs(n_sec_a, bounds_a, n_sec_b, bounds_b, pair_offset, t->dimension[leg]));
  cudaStream_t s = (cudaStream_t)stream;
  TQ_CHECK(sync_device_meta(const_cast<tq_bs *>(t), s));
  std::vector<int64_t> dim;
  for (int32_t l = 0; l < t->rank; l++) {
    if (l == leg) {
      dim.push_back(bounds_a[n_sec_a]);
      dim.push_back(bounds_b[n_sec_b]);
    } else {
      dim.push_back(t->dimension[l]);
    }
  }
  tq_bs *C = new_tensor(t->dtype, t->rank + 1, dim.data());
  std::unique_ptr<tq_bs, tq_status (*)(tq_bs *)> guard(C, tq_bs_destroy);
  const int64_t nb = t->nb, nr = t->rank + 1, np = n_sec_a * n_sec_b;
  C->nb = nb;
  TQ_CHECK(C->d_meta.alloc(3 * (size_t)nb * nr + nb, s));
  // pair starts in ascending order with their pair index
  std::vector<std::pair<int64_t, int64_t>> st;
  for (int64_t q = 0; q < np; q++) st.push_back({pair_offset[q], q});
  std::sort(st.begin(), st.end());
  std::vector<int64_t> h(bounds_a, bounds_a + n_sec_a + 1);
  h.insert(h.end(), bounds_b, bounds_b + n_sec_b + 1);
  for (auto &x : st) h.push_back(x.first);
  for (auto &x : st) h.push_back(x.second);
  DevArray<int64_t> tab;
  DevArray<int32_t> bad;
  TQ_CHECK(tab.alloc(h.size(), s));
  TQ_CHECK(bad.alloc(1, s));
  TQ_CUDA(cudaMemcpyAsync(tab.p, h.data(), h.size() * 8, cudaMemcpyHostToDevice, s));
  TQ_CUDA(cudaMemsetAsync(bad.p, 0, 4, s));
  const DevBS v = t->view();
  int64_t *nbeg = C->d_meta.p, *nend = nbeg + nb * nr, *nstr = nend + nb * nr, *noff = nstr + nb * nr;
  if (nb) {
    const int64_t *ta = tab.p, *tb = ta + n_sec_a + 1, *ps = tb + n_sec_b + 1, *pi = ps + np;
    count_launch(), split_kernel<<<(unsigned)((nb + 255) / 256), 256, 0, s>>>(
        v, leg, ta, n_sec_a, tb, ps, pi, np, nbeg, nend, nstr, bad.p);
    TQ_CUDA(cudaGetLastError());
    TQ_CUDA(cudaMemcpyAsync(noff, v.offsets, nb * 8, cudaMemcpyDeviceToDevice, s));
  }
  TQ_CHECK(alloc_data(C, t->n_elem, s));
  if (t->n_elem)
    TQ_CUDA(cudaMemcpyAsync(C->data, t->data, t->n_elem * dtype_size(t->dtype),
                            cudaMemcpyDeviceToDevice, s));
  int32_t h_bad = 0;
  TQ_CUDA(cudaMemcpyAsync(&h_bad, bad.p, 4, cudaMemcpyDeviceToHost, s));
  TQ_CUDA(cudaStreamSynchronize(s));  // h (host staging) and h_bad
  if (h_bad)
    return fail(TQ_ERR_UNSUPPORTED,
                "split_leg needs every block to cover exactly one sector pair of the fused leg");
  C->host_valid = false;
  C->dev_valid = true;
  *out = guard.release();
  return TQ_OK;
}


tq_status tq_bs_fuse_legs(const tq_bs *t, int32_t leg, int64_t n_sec_a, const int64_t *bounds_a,
                          int64_t n_sec_b, const int64_t *bounds_b, const int64_t *pair_offset,
                          tq_stream stream, tq_bs **out) {
  if (!t || !out || !bounds_a || !bounds_b || !pair_offset)
    return fail(TQ_ERR_INVALID, "NULL argument");
  if (leg < 0 || leg + 1 >= t->rank) return fail(TQ_ERR_INVALID, "legs to fuse out of range");
  if (n_sec_a <= 0 || n_sec_b <= 0) return fail(TQ_ERR_INVALID, "empty sector list");
  if (bounds_a[0] != 0 || bounds_a[n_sec_a] != t->dimension[leg] || bounds_b[0] != 0 ||
      bounds_b[n_sec_b] != t->dimension[leg + 1])
    return fail(TQ_ERR_INVALID, "sector bounds do not span the legs");
  const int64_t fused = t->dimension[leg] * t->dimension[leg + 1];
  TQ_CHECK(check_pairs(n_sec_a, bounds_a, n_sec_b, bounds_b, pair_offset, fused));
  cudaStream_t s = (cudaStream_t)stream;
  TQ_CHECK(sync_device_meta(const_cast<tq_bs *>(t), s));
  std::vector<int64_t> dim;
  for (int32_t l = 0; l < t->rank; l++) {
    if (l == leg + 1) continue;
    dim.push_back(l == leg ? fused : t->dimension[l]);
  }
  tq_bs *C = new_tensor(t->dtype, t->rank - 1, dim.data());
  std::unique_ptr<tq_bs, tq_status (*)(tq_bs *)> guard(C, tq_bs_destroy);
  const int64_t nb = t->nb, nr = t->rank - 1;
  C->nb = nb;
  TQ_CHECK(C->d_meta.alloc(3 * (size_t)nb * nr + nb, s));
  DevArray<int64_t> tab;
  DevArray<int32_t> bad;
  TQ_CHECK(tab.alloc((n_sec_a + 1) + (n_sec_b + 1) + n_sec_a * n_sec_b, s));
  TQ_CHECK(bad.alloc(1, s));
  std::vector<int64_t> h(bounds_a, bounds_a + n_sec_a + 1);
  h.insert(h.end(), bounds_b, bounds_b + n_sec_b + 1);
  h.insert(h.end(), pair_offset, pair_offset + n_sec_a * n_sec_b);
  TQ_CUDA(cudaMemcpyAsync(tab.p, h.data(), h.size() * 8, cudaMemcpyHostToDevice, s));
  TQ_CUDA(cudaMemsetAsync(bad.p, 0, 4, s));
  const DevBS v = t->view();
  int64_t *nbeg = C->d_meta.p, *nend = nbeg + nb * nr, *nstr = nend + nb * nr, *noff = nstr + nb * nr;
  if (nb) {
    count_launch(), fuse_kernel<<<(unsigned)((nb + 255) / 256), 256, 0, s>>>(
        v, leg, tab.p, n_sec_a, tab.p + n_sec_a + 1, n_sec_b, tab.p + n_sec_a + n_sec_b + 2, nbeg,
        nend, nstr, bad.p);
    TQ_CUDA(cudaGetLastError());
    TQ_CUDA(cudaMemcpyAsync(noff, v.offsets, nb * 8, cudaMemcpyDeviceToDevice, s));
  }
  TQ_CHECK(alloc_data(C, t->n_elem, s));
  if (t->n_elem)
    TQ_CUDA(cudaMemcpyAsync(C->data, t->data, t->n_elem * dtype_size(t->dtype),
                            cudaMemcpyDeviceToDevice, s));
  int32_t h_bad = 0;
  TQ_CUDA(cudaMemcpyAsync(&h_bad, bad.p, 4, cudaMemcpyDeviceToHost, s));
  TQ_CUDA(cudaStreamSynchronize(s));  // h (host staging) and h_bad
  if (h_bad)
    return fail(TQ_ERR_UNSUPPORTED,
                "fuse_legs needs every block to cover whole sectors of both legs, with "
                "contiguous strides across them");
  C->host_valid = false;
  C->dev_valid = true;
  *out = guard.release();
  return TQ_OK;
}

}  // extern "C"
