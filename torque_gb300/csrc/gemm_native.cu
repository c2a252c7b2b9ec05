// Native-precision grouped block GEMM (the drop-in arithmetic).
//
// GB300 runs FP64 at about 1/1800 of its bf16 tensor rate, so this kernel is
// bound by the FP64 pipe at a few flop per byte; a 64x64x16 register-blocked
// SIMT tile with operands staged in shared memory reaches that bound without
// tensor cores (tcgen05 has no f64 kind).  One CTA per output tile; the CTA
// walks the pairs of its output block in reference order and accumulates
// them in registers, which is the FP64 summation of block-pair partials.
#include <cuda_fp16.h>

#include "gemm.cuh"

namespace tq {

// Element type T is stored; Acc accumulates (binary16 accumulates in FP32).
__device__ __forceinline__ double to_acc(double x) { return x; }
__device__ __forceinline__ float to_acc(float x) { return x; }
__device__ __forceinline__ float to_acc(__half x) { return __half2float(x); }
template <typename T> __device__ __forceinline__ T from_acc(double x) { return (T)x; }
template <typename T> __device__ __forceinline__ T from_acc(float x) { return (T)x; }
template <> __device__ __forceinline__ __half from_acc<__half>(float x) { return __float2half_rn(x); }

__device__ __forceinline__ int64_t find_seg(const int64_t *start, int64_t n, int64_t t) {
  // largest o with start[o] <= t (start is non-decreasing, start[0] = 0)
  int64_t lo = 0, hi = n - 1;
  while (lo < hi) {
    const int64_t mid = (lo + hi + 1) >> 1;
    if (start[mid] <= t) lo = mid; else hi = mid - 1;
  }
  return lo;
}

template <typename T, typename Acc>
__device__ __forceinline__ void load_tile(const T *__restrict__ data, const Operand &op,
                                          int64_t r0, int64_t k0, int64_t kmax,
                                          Acc (*S)[NT_TM + 1]) {
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
    Acc v = Acc(0);
    if (gr < op.rows && gk < kmax) {
      int64_t a;
      if (rs >= 0 && cs >= 0) a = op.base + gr * rs + gk * cs;
      else a = op.base + mixed_addr(gr, op.nr, op.rdim, op.rst) + mixed_addr(gk, op.nc, op.cdim, op.cst);
      v = to_acc(data[a]);
    }
    S[kk][r] = v;
  }
}

// Rows and columns of output o (from its first pair).
__device__ __forceinline__ void out_dims(const GemmJob &job, int64_t o, int64_t &m, int64_t &n) {
  const int64_t p0 = job.perm ? job.perm[job.seg[o]] : job.seg[o];
  const int64_t i = job.pa[p0], j = job.pb[p0];
  m = 1;
  n = 1;
  for (int q = 0; q < job.L.nfa; q++)
    m *= job.A.end[i * job.A.rank + job.L.fa[q]] - job.A.begin[i * job.A.rank + job.L.fa[q]] + 1;
  for (int q = 0; q < job.L.nfb; q++)
    n *= job.B.end[j * job.B.rank + job.L.fb[q]] - job.B.begin[j * job.B.rank + job.L.fb[q]] + 1;
}

// One CTA per work item: an output tile, or one K chunk of it (split-K).  A
// chunk covers a contiguous range of the output's fused K (its pairs' columns
// back to back, in pair order); chunk boundaries fall on multiples of 16.
template <typename T, typename Acc>
__global__ void __launch_bounds__(NT_THREADS) gemm_native_kernel(GemmJob job, int64_t tile_base) {
  __shared__ Acc As[NT_TK][NT_TM + 1];
  __shared__ Acc Bs[NT_TK][NT_TN + 1];
  __shared__ Operand opA, opB;
  __shared__ int64_t s_o, s_tm, s_tn, s_tile, s_klo, s_khi;
  __shared__ int32_t s_c, s_ch;
  const int t = threadIdx.x, tx = t & 15, ty = t >> 4;
  const int64_t tile = tile_base + blockIdx.x;
  if (t == 0) {
    const int64_t o = find_seg(job.tile_start, job.n_out, tile);
    s_o = o;
    int64_t m, n;
    out_dims(job, o, m, n);
    const int64_t tiles_m = (m + NT_TM - 1) / NT_TM;
    int64_t local = tile - job.tile_start[o];
    const int32_t ch = job.chunks ? job.chunks[o] : 1;
    const int32_t c = (int32_t)(local % ch);
    local /= ch;
    s_tile = local;
    s_tm = local % tiles_m;
    s_tn = local / tiles_m;
    s_c = c;
    s_ch = ch;
    if (ch > 1) {
      const int64_t kf = job.kfused[o];
      s_klo = (kf * c / ch) & ~(int64_t)15;
      s_khi = c + 1 == ch ? kf : (kf * (c + 1) / ch) & ~(int64_t)15;
    } else {
      s_klo = 0;
      s_khi = INT64_MAX;
    }
  }
  __syncthreads();
  const int64_t o = s_o, r0 = s_tm * NT_TM, c0 = s_tn * NT_TN, klo = s_klo, khi = s_khi;
  const T *Ad = (const T *)job.A.data;
  const T *Bd = (const T *)job.B.data;
  Acc acc[4][4];
#pragma unroll
  for (int a = 0; a < 4; a++)
#pragma unroll
    for (int b = 0; b < 4; b++) acc[a][b] = Acc(0);

  int64_t pos = 0;  // fused-K column of the current pair's first column
  for (int64_t sidx = job.seg[o]; sidx < job.seg[o + 1] && pos < khi; sidx++) {
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
    const int64_t kb = klo > pos ? klo - pos : 0;
    const int64_t ke = khi - pos < K ? khi - pos : K;
    for (int64_t k0 = kb; k0 < ke; k0 += NT_TK) {
      load_tile<T, Acc>(Ad, opA, r0, k0, ke, As);
      load_tile<T, Acc>(Bd, opB, c0, k0, ke, Bs);
      __syncthreads();
#pragma unroll
      for (int kk = 0; kk < NT_TK; kk++) {
        Acc a[4], b[4];
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
    pos += K;
    __syncthreads();  // every thread has read opA.cols before the next pair's operands
  }
  if (s_ch > 1) {
    // partial tile, full 64x64, in chunk order after the tile's other chunks
    Acc *P = (Acc *)job.scratch + (job.split_off[o] + s_tile * s_ch + s_c) * (int64_t)(NT_TM * NT_TN);
#pragma unroll
    for (int y = 0; y < 4; y++)
#pragma unroll
      for (int x = 0; x < 4; x++) P[(tx + 16 * x) + (ty + 16 * y) * NT_TM] = acc[x][y];
    return;
  }
  int64_t m, n;
  out_dims(job, o, m, n);
  T *C = (T *)job.C + job.c_off[o];
#pragma unroll
  for (int y = 0; y < 4; y++) {
    const int64_t c = c0 + ty + 16 * y;
    if (c >= n) continue;
#pragma unroll
    for (int x = 0; x < 4; x++) {
      const int64_t r = r0 + tx + 16 * x;
      if (r < m) C[r + c * m] = from_acc<T>(acc[x][y]);
    }
  }
}

// Split tiles: C tile = sum of its chunk partials in chunk order.
template <typename T, typename Acc>
__global__ void __launch_bounds__(NT_THREADS) split_reduce_kernel(GemmJob job,
                                                                  const int64_t *split_start,
                                                                  int64_t base) {
  const int64_t st = base + blockIdx.x;
  const int64_t o = find_seg(split_start, job.n_out, st);
  const int64_t local = st - split_start[o];
  int64_t m, n;
  out_dims(job, o, m, n);
  const int64_t tiles_m = (m + NT_TM - 1) / NT_TM;
  const int64_t r0 = (local % tiles_m) * NT_TM, c0 = (local / tiles_m) * NT_TN;
  const int ch = job.chunks[o];
  const Acc *P = (const Acc *)job.scratch + (job.split_off[o] + local * ch) * (int64_t)(NT_TM * NT_TN);
  T *C = (T *)job.C + job.c_off[o];
  for (int e = threadIdx.x; e < NT_TM * NT_TN; e += NT_THREADS) {
    const int64_t r = r0 + e % NT_TM, c = c0 + e / NT_TM;
    if (r >= m || c >= n) continue;
    Acc v = P[e];
    for (int q = 1; q < ch; q++) v += P[(int64_t)q * NT_TM * NT_TN + e];
    C[r + c * m] = from_acc<T>(v);
  }
}

tq_status launch_gemm_native(const GemmJob &job_in, int64_t n_tiles, tq_dtype dt, cudaStream_t s,
                             const NativeWork *w) {
  GemmJob job = job_in;
  if (w && w->chunks) {
    job.tile_start = w->work_start;
    job.chunks = w->chunks;
    job.split_off = w->split_off;
    job.kfused = w->kfused;
    job.scratch = w->scratch;
    n_tiles = w->n_work;
  }
  const int64_t max_grid = 0x7fffffff;
  for (int64_t base = 0; base < n_tiles; base += max_grid) {
    const unsigned g = (unsigned)std::min<int64_t>(max_grid, n_tiles - base);
    if (dt == TQ_F64)
      count_launch(), gemm_native_kernel<double, double><<<g, NT_THREADS, 0, s>>>(job, base);
    else if (dt == TQ_F32)
      count_launch(), gemm_native_kernel<float, float><<<g, NT_THREADS, 0, s>>>(job, base);
    else
      count_launch(), gemm_native_kernel<__half, float><<<g, NT_THREADS, 0, s>>>(job, base);
    TQ_CUDA(cudaGetLastError());
  }
  if (w && w->chunks) {
    for (int64_t base = 0; base < w->n_split; base += max_grid) {
      const unsigned g = (unsigned)std::min<int64_t>(max_grid, w->n_split - base);
      if (dt == TQ_F64)
        count_launch(), split_reduce_kernel<double, double><<<g, NT_THREADS, 0, s>>>(job, w->split_start, base);
      else if (dt == TQ_F32)
        count_launch(), split_reduce_kernel<float, float><<<g, NT_THREADS, 0, s>>>(job, w->split_start, base);
      else
        count_launch(), split_reduce_kernel<__half, float><<<g, NT_THREADS, 0, s>>>(job, w->split_start, base);
      TQ_CUDA(cudaGetLastError());
    }
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

template <typename T, typename Acc>
__global__ void __launch_bounds__(NT_THREADS) dot_chunks_kernel(GemmJob job, int64_t n_pairs,
                                                                 const int64_t *chunk_start,
                                                                 Acc *partials) {
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
  Acc acc = Acc(0);
  for (int64_t k = s_k0 + threadIdx.x; k < k_end; k += NT_THREADS)
    acc = fma(to_acc(Ad[opA.base + mixed_addr(k, opA.nc, opA.cdim, opA.cst)]),
              to_acc(Bd[opB.base + mixed_addr(k, opB.nc, opB.cdim, opB.cst)]), acc);
  const Acc s = block_sum_fixed<Acc>(acc);
  if (threadIdx.x == 0) partials[c] = s;
}

template <typename T, typename Acc>
__global__ void __launch_bounds__(NT_THREADS) sum_partials_kernel(const Acc *partials, int64_t n,
                                                                   T *out) {
  Acc acc = Acc(0);
  for (int64_t q = threadIdx.x; q < n; q += NT_THREADS) acc += partials[q];
  const Acc s = block_sum_fixed<Acc>(acc);
  if (threadIdx.x == 0) *out = from_acc<T>(s);
}

tq_status launch_dot_native(const GemmJob &job, int64_t n_pairs, const int64_t *chunk_start,
                            int64_t n_chunks, void *partials, tq_dtype dt, cudaStream_t s) {
  if (n_chunks == 0) {
    TQ_CUDA(cudaMemsetAsync(job.C, 0, dtype_size(dt), s));
    return TQ_OK;
  }
  const unsigned g = (unsigned)n_chunks;
  if (dt == TQ_F64) {
    count_launch(), dot_chunks_kernel<double, double><<<g, NT_THREADS, 0, s>>>(
        job, n_pairs, chunk_start, (double *)partials);
    count_launch(), sum_partials_kernel<double, double><<<1, NT_THREADS, 0, s>>>(
        (const double *)partials, n_chunks, (double *)job.C);
  } else if (dt == TQ_F32) {
    count_launch(), dot_chunks_kernel<float, float><<<g, NT_THREADS, 0, s>>>(
        job, n_pairs, chunk_start, (float *)partials);
    count_launch(), sum_partials_kernel<float, float><<<1, NT_THREADS, 0, s>>>(
        (const float *)partials, n_chunks, (float *)job.C);
  } else {
    count_launch(), dot_chunks_kernel<__half, float><<<g, NT_THREADS, 0, s>>>(
        job, n_pairs, chunk_start, (float *)partials);
    count_launch(), sum_partials_kernel<__half, float><<<1, NT_THREADS, 0, s>>>(
        (const float *)partials, n_chunks, (__half *)job.C);
  }
  TQ_CUDA(cudaGetLastError());
  return TQ_OK;
}

}  // namespace tq
