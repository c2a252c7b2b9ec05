// Native-precision grouped block GEMM (the drop-in arithmetic).
//
// GB300 runs FP64 at about 1/1800 of its bf16 tensor rate, so this kernel is
// bound by the FP64 pipe at a few flop per byte; a 64x64x16 register-blocked
// SIMT tile with operands staged in shared memory reaches that bound without
// tensor cores (tcgen05 has no f64 kind).  One CTA per output tile; the CTA
// walks the pairs of its output block in reference order and accumulates
// them in registers, which is the FP64 summation of block-pair partials.
#include "gemm.cuh"

namespace tq {

__device__ __forceinline__ int64_t find_seg(const int64_t *start, int64_t n, int64_t t) {
  // largest o with start[o] <= t (start is non-decreasing, start[0] = 0)
  int64_t lo = 0, hi = n - 1;
  while (lo < hi) {
    const int64_t mid = (lo + hi + 1) >> 1;
    if (start[mid] <= t) lo = mid; else hi = mid - 1;
  }
  return lo;
}

template <typename T>
__device__ __forceinline__ void load_tile(const T *__restrict__ data, const Operand &op,
                                          int64_t r0, int64_t k0, T (*S)[NT_TM + 1]) {
  const int64_t rs = row_stride(op), cs = col_stride(op);
  const int t = threadIdx.x;
  const bool m_major = rs == 1 || (rs != -1 && cs != 1);
#pragma unroll
  for (int q = 0; q < (NT_TM * NT_TK) / NT_THREADS; q++) {
    const int e = t + q * NT_THREADS;
    int r, kk;
    if (m_major) { r = e % NT_TM; kk = e / NT_TM; }
    else { kk = e % NT_TK; r = e / NT_TK; }
    const int64_t gr = r0 + r, gk = k0 + kk;
    T v = T(0);
    if (gr < op.rows && gk < op.cols) {
      int64_t a;
      if (rs >= 0 && cs >= 0) a = op.base + gr * rs + gk * cs;
      else a = op.base + mixed_addr(gr, op.nr, op.rdim, op.rst) + mixed_addr(gk, op.nc, op.cdim, op.cst);
      v = data[a];
    }
    S[kk][r] = v;
  }
}

template <typename T>
__global__ void __launch_bounds__(NT_THREADS) gemm_native_kernel(GemmJob job, int64_t tile_base) {
  __shared__ T As[NT_TK][NT_TM + 1];
  __shared__ T Bs[NT_TK][NT_TN + 1];
  __shared__ Operand opA, opB;
  __shared__ int64_t s_o, s_tm, s_tn;
  const int t = threadIdx.x, tx = t & 15, ty = t >> 4;
  const int64_t tile = tile_base + blockIdx.x;
  if (t == 0) {
    const int64_t o = find_seg(job.tile_start, job.n_out, tile);
    s_o = o;
    // rows/cols of the output block come from its first pair
    const int64_t p0 = job.perm ? job.perm[job.seg[o]] : job.seg[o];
    const int64_t i = job.pa[p0], j = job.pb[p0];
    int64_t m = 1, n = 1;
    for (int q = 0; q < job.L.nfa; q++)
      m *= job.A.end[i * job.A.rank + job.L.fa[q]] - job.A.begin[i * job.A.rank + job.L.fa[q]] + 1;
    for (int q = 0; q < job.L.nfb; q++)
      n *= job.B.end[j * job.B.rank + job.L.fb[q]] - job.B.begin[j * job.B.rank + job.L.fb[q]] + 1;
    const int64_t tiles_m = (m + NT_TM - 1) / NT_TM;
    const int64_t local = tile - job.tile_start[o];
    s_tm = local % tiles_m;
    s_tn = local / tiles_m;
  }
  __syncthreads();
  const int64_t o = s_o, r0 = s_tm * NT_TM, c0 = s_tn * NT_TN;
  const T *Ad = (const T *)job.A.data;
  const T *Bd = (const T *)job.B.data;
  T acc[4][4];
#pragma unroll
  for (int a = 0; a < 4; a++)
#pragma unroll
    for (int b = 0; b < 4; b++) acc[a][b] = T(0);

  for (int64_t sidx = job.seg[o]; sidx < job.seg[o + 1]; sidx++) {
    const int64_t p = job.perm ? job.perm[sidx] : sidx;
    if (t == 0 || t == 32) {
      const int64_t i = job.pa[p], j = job.pb[p];
      int64_t cb[TQ_MAXR], ce[TQ_MAXR];
      contraction_range(job.A, job.B, job.L, i, j, cb, ce);
      if (t == 0)
        build_operand(job.A, i, job.L.nfa, job.L.fa, job.L.nc, job.L.al, cb, ce, opA);
      else
        build_operand(job.B, j, job.L.nfb, job.L.fb, job.L.nc, job.L.bl, cb, ce, opB);
    }
    __syncthreads();
    const int64_t K = opA.cols;
    for (int64_t k0 = 0; k0 < K; k0 += NT_TK) {
      load_tile<T>(Ad, opA, r0, k0, As);
      load_tile<T>(Bd, opB, c0, k0, Bs);
      __syncthreads();
#pragma unroll
      for (int kk = 0; kk < NT_TK; kk++) {
        T a[4], b[4];
#pragma unroll
        for (int q = 0; q < 4; q++) {
          a[q] = As[kk][tx + 16 * q];
          b[q] = Bs[kk][ty + 16 * q];
        }
#pragma unroll
        for (int x = 0; x < 4; x++)
#pragma unroll
          for (int y = 0; y < 4; y++) acc[x][y] = fma(a[x], b[y], acc[x][y]);
      }
      __syncthreads();
    }
  }
  const int64_t m = opA.rows, n = opB.rows;
  T *C = (T *)job.C + job.c_off[o];
#pragma unroll
  for (int y = 0; y < 4; y++) {
    const int64_t c = c0 + ty + 16 * y;
    if (c >= n) continue;
#pragma unroll
    for (int x = 0; x < 4; x++) {
      const int64_t r = r0 + tx + 16 * x;
      if (r < m) C[r + c * m] = acc[x][y];
    }
  }
}

tq_status launch_gemm_native(const GemmJob &job, int64_t n_tiles, tq_dtype dt, cudaStream_t s) {
  const int64_t max_grid = 0x7fffffff;
  for (int64_t base = 0; base < n_tiles; base += max_grid) {
    const unsigned g = (unsigned)std::min<int64_t>(max_grid, n_tiles - base);
    if (dt == TQ_F64)
      count_launch(), gemm_native_kernel<double><<<g, NT_THREADS, 0, s>>>(job, base);
    else
      count_launch(), gemm_native_kernel<float><<<g, NT_THREADS, 0, s>>>(job, base);
    TQ_CUDA(cudaGetLastError());
  }
  return TQ_OK;
}

// ---------------------------------------------------------------- rank-0 path
template <typename T>
__device__ __forceinline__ T block_sum_fixed(T v) {
  __shared__ T red[NT_THREADS];
  red[threadIdx.x] = v;
  __syncthreads();
  for (int w = NT_THREADS / 2; w > 0; w >>= 1) {
    if (threadIdx.x < w) red[threadIdx.x] += red[threadIdx.x + w];
    __syncthreads();
  }
  T r = red[0];
  __syncthreads();
  return r;
}

template <typename T>
__global__ void __launch_bounds__(NT_THREADS) dot_chunks_kernel(GemmJob job, int64_t n_pairs,
                                                                 const int64_t *chunk_start,
                                                                 T *partials) {
  __shared__ Operand opA, opB;
  __shared__ int64_t s_k0;
  const int64_t c = blockIdx.x;
  if (threadIdx.x == 0 || threadIdx.x == 32) {
    const int64_t p = find_seg(chunk_start, n_pairs, c);
    const int64_t i = job.pa[p], j = job.pb[p];
    int64_t cb[TQ_MAXR], ce[TQ_MAXR];
    contraction_range(job.A, job.B, job.L, i, j, cb, ce);
    if (threadIdx.x == 0) {
      build_operand(job.A, i, 0, job.L.fa, job.L.nc, job.L.al, cb, ce, opA);
      s_k0 = (c - chunk_start[p]) * DOT_CHUNK;
    } else {
      build_operand(job.B, j, 0, job.L.fb, job.L.nc, job.L.bl, cb, ce, opB);
    }
  }
  __syncthreads();
  const T *Ad = (const T *)job.A.data;
  const T *Bd = (const T *)job.B.data;
  const int64_t k_end = min(opA.cols, s_k0 + DOT_CHUNK);
  T acc = T(0);
  for (int64_t k = s_k0 + threadIdx.x; k < k_end; k += NT_THREADS)
    acc = fma(Ad[opA.base + mixed_addr(k, opA.nc, opA.cdim, opA.cst)],
              Bd[opB.base + mixed_addr(k, opB.nc, opB.cdim, opB.cst)], acc);
  const T s = block_sum_fixed<T>(acc);
  if (threadIdx.x == 0) partials[c] = s;
}

template <typename T>
__global__ void __launch_bounds__(NT_THREADS) sum_partials_kernel(const T *partials, int64_t n,
                                                                   T *out) {
  T acc = T(0);
  for (int64_t q = threadIdx.x; q < n; q += NT_THREADS) acc += partials[q];
  const T s = block_sum_fixed<T>(acc);
  if (threadIdx.x == 0) *out = s;
}

tq_status launch_dot_native(const GemmJob &job, int64_t n_pairs, const int64_t *chunk_start,
                            int64_t n_chunks, void *partials, tq_dtype dt, cudaStream_t s) {
  if (n_chunks == 0) {
    TQ_CUDA(cudaMemsetAsync(job.C, 0, dtype_size(dt), s));
    return TQ_OK;
  }
  if (dt == TQ_F64) {
    count_launch(), dot_chunks_kernel<double><<<(unsigned)n_chunks, NT_THREADS, 0, s>>>(job, n_pairs, chunk_start,
                                                                        (double *)partials);
    count_launch(), sum_partials_kernel<double><<<1, NT_THREADS, 0, s>>>((const double *)partials, n_chunks,
                                                         (double *)job.C);
  } else {
    count_launch(), dot_chunks_kernel<float><<<(unsigned)n_chunks, NT_THREADS, 0, s>>>(job, n_pairs, chunk_start,
                                                                       (float *)partials);
    count_launch(), sum_partials_kernel<float><<<1, NT_THREADS, 0, s>>>((const float *)partials, n_chunks,
                                                        (float *)job.C);
  }
  TQ_CUDA(cudaGetLastError());
  return TQ_OK;
}

}  // namespace tq
