// Batched dense algebra on per-vesicle blocks: tiled GEMM (FP64/FP32),
// GEMV, blocked LU with partial pivoting and LU solve, and the deterministic
// dot-product reduction used by GMRES.
#include "ves_internal.h"

// ----------------------------------------------------------------------------
// C[b] = alpha * A[b] (MxK) * B[b] (KxN) + beta * C[b], row-major, 64x64 tiles.
template <typename T>
__global__ void __launch_bounds__(256) bgemm_kernel(int M, int N, int K, T alpha, const T* __restrict__ A,
                                                    int lda, long long sA, const T* __restrict__ B, int ldb,
                                                    long long sB, T beta, T* __restrict__ C, int ldc,
                                                    long long sC) {
  constexpr int TM = 64, TN = 64, TK = 16;
  __shared__ T As[TK][TM + 1];
  __shared__ T Bs[TK][TN];
  const long long b = blockIdx.z;
  const T* Ab = A + b * sA;
  const T* Bb = B + b * sB;
  T* Cb = C + b * sC;
  const int row0 = blockIdx.y * TM, col0 = blockIdx.x * TN;
  const int tx = threadIdx.x % 16, ty = threadIdx.x / 16;  // 16x16 threads, 4x4 outputs each
  T acc[4][4];
#pragma unroll
  for (int i = 0; i < 4; ++i)
#pragma unroll
    for (int j = 0; j < 4; ++j) acc[i][j] = T(0);
  for (int k0 = 0; k0 < K; k0 += TK) {
    for (int idx = threadIdx.x; idx < TM * TK; idx += 256) {
      const int r = idx / TK, kk = idx % TK;
      const int gr = row0 + r, gk = k0 + kk;
      As[kk][r] = (gr < M && gk < K) ? Ab[(long long)gr * lda + gk] : T(0);
    }
    for (int idx = threadIdx.x; idx < TK * TN; idx += 256) {
      const int kk = idx / TN, cc = idx % TN;
      const int gk = k0 + kk, gc = col0 + cc;
      Bs[kk][cc] = (gk < K && gc < N) ? Bb[(long long)gk * ldb + gc] : T(0);
    }
    __syncthreads();
#pragma unroll
    for (int kk = 0; kk < TK; ++kk) {
      T a[4], bb[4];
#pragma unroll
      for (int i = 0; i < 4; ++i) a[i] = As[kk][ty * 4 + i];
#pragma unroll
      for (int j = 0; j < 4; ++j) bb[j] = Bs[kk][tx * 4 + j];
#pragma unroll
      for (int i = 0; i < 4; ++i)
#pragma unroll
        for (int j = 0; j < 4; ++j) acc[i][j] = fma(a[i], bb[j], acc[i][j]);
    }
    __syncthreads();
  }
#pragma unroll
  for (int i = 0; i < 4; ++i) {
    const int gr = row0 + ty * 4 + i;
    if (gr >= M) continue;
#pragma unroll
    for (int j = 0; j < 4; ++j) {
      const int gc = col0 + tx * 4 + j;
      if (gc >= N) continue;
      T* cp = Cb + (long long)gr * ldc + gc;
      *cp = (beta == T(0)) ? alpha * acc[i][j] : fma(alpha, acc[i][j], beta * *cp);
    }
  }
}

// FP32 variant for aligned shapes: 128x128 tiles, K steps of 8, 8x8 outputs
// per thread (rows ty*4+i and 64+ty*4+i, columns tx*4+j and 64+tx*4+j), 16-byte
// operand loads.  Needs K % 8 == 0, N % 4 == 0, lda/ldb/sA/sB multiples of 4
// and 16-byte aligned A and B.
__global__ void __launch_bounds__(256) bgemm128_f32_kernel(int M, int N, int K, float alpha,
                                                           const float* __restrict__ A, int lda, long long sA,
                                                           const float* __restrict__ B, int ldb, long long sB,
                                                           float beta, float* __restrict__ C, int ldc,
                                                           long long sC) {
  constexpr int TK = 8, LDS = 132;  // padded rows: the transposed A stores are conflict-free
  __shared__ __align__(16) float As[TK][LDS];
  __shared__ __align__(16) float Bs[TK][LDS];
  const long long b = blockIdx.z;
  const float* Ab = A + b * sA;
  const float* Bb = B + b * sB;
  float* Cb = C + b * sC;
  const int row0 = blockIdx.y * 128, col0 = blockIdx.x * 128;
  const int t = threadIdx.x, tx = t % 16, ty = t / 16;
  // load assignments: A row t/2, k chunk (t%2)*4; B row t/32, columns (t%32)*4
  const int ar = t >> 1, ak = (t & 1) * 4;
  const int bk = t >> 5, bc = (t & 31) * 4;
  const bool arow_ok = row0 + ar < M;
  const bool bcol_ok = col0 + bc < N;  // N % 4 == 0: the whole float4 is in range
  float acc[8][8];
#pragma unroll
  for (int i = 0; i < 8; ++i)
#pragma unroll
    for (int j = 0; j < 8; ++j) acc[i][j] = 0.f;
  for (int k0 = 0; k0 < K; k0 += TK) {
    const float4 av = arow_ok ? *reinterpret_cast<const float4*>(Ab + (long long)(row0 + ar) * lda + k0 + ak)
                              : make_float4(0.f, 0.f, 0.f, 0.f);
    const float4 bv = bcol_ok ? *reinterpret_cast<const float4*>(Bb + (long long)(k0 + bk) * ldb + col0 + bc)
                              : make_float4(0.f, 0.f, 0.f, 0.f);
    __syncthreads();
    As[ak + 0][ar] = av.x;
    As[ak + 1][ar] = av.y;
    As[ak + 2][ar] = av.z;
    As[ak + 3][ar] = av.w;
    *reinterpret_cast<float4*>(&Bs[bk][bc]) = bv;
    __syncthreads();
#pragma unroll
    for (int kk = 0; kk < TK; ++kk) {
      const float4 a0 = *reinterpret_cast<const float4*>(&As[kk][ty * 4]);
      const float4 a1 = *reinterpret_cast<const float4*>(&As[kk][64 + ty * 4]);
      const float4 b0 = *reinterpret_cast<const float4*>(&Bs[kk][tx * 4]);
      const float4 b1 = *reinterpret_cast<const float4*>(&Bs[kk][64 + tx * 4]);
      const float a[8] = {a0.x, a0.y, a0.z, a0.w, a1.x, a1.y, a1.z, a1.w};
      const float bb[8] = {b0.x, b0.y, b0.z, b0.w, b1.x, b1.y, b1.z, b1.w};
#pragma unroll
      for (int i = 0; i < 8; ++i)
#pragma unroll
        for (int j = 0; j < 8; ++j) acc[i][j] = fmaf(a[i], bb[j], acc[i][j]);
    }
  }
#pragma unroll
  for (int i = 0; i < 8; ++i) {
    const int gr = row0 + (i < 4 ? ty * 4 + i : 64 + ty * 4 + i - 4);
    if (gr >= M) continue;
#pragma unroll
    for (int j = 0; j < 8; ++j) {
      const int gc = col0 + (j < 4 ? tx * 4 + j : 64 + tx * 4 + j - 4);
      if (gc >= N) continue;
      float* cp = Cb + (long long)gr * ldc + gc;
      *cp = (beta == 0.f) ? alpha * acc[i][j] : fmaf(alpha, acc[i][j], beta * *cp);
    }
  }
}

template <typename T>
static void bgemm_launch(int batch, int M, int N, int K, T alpha, const T* A, int lda, long long sA,
                         const T* B, int ldb, long long sB, T beta, T* C, int ldc, long long sC,
                         cudaStream_t s) {
  for (int b0 = 0; b0 < batch; b0 += 65535) {
    const int nb = batch - b0 < 65535 ? batch - b0 : 65535;
    dim3 grid(ceil_div(N, 64), ceil_div(M, 64), nb);
    ves_count_launch();
    bgemm_kernel<T><<<grid, 256, 0, s>>>(M, N, K, alpha, A + b0 * sA, lda, sA, B + b0 * sB, ldb, sB, beta,
                                         C + b0 * sC, ldc, sC);
  }
}

void launch_bgemm_f64(int batch, int M, int N, int K, double alpha, const double* A, int lda,
                      long long sA, const double* B, int ldb, long long sB, double beta, double* C,
                      int ldc, long long sC, cudaStream_t s) {
  bgemm_launch<double>(batch, M, N, K, alpha, A, lda, sA, B, ldb, sB, beta, C, ldc, sC, s);
}
void launch_bgemm_f32(int batch, int M, int N, int K, float alpha, const float* A, int lda,
                      long long sA, const float* B, int ldb, long long sB, float beta, float* C,
                      int ldc, long long sC, cudaStream_t s) {
  const bool aligned = K % 8 == 0 && N % 4 == 0 && lda % 4 == 0 && ldb % 4 == 0 && sA % 4 == 0 && sB % 4 == 0 &&
                       ((reinterpret_cast<uintptr_t>(A) | reinterpret_cast<uintptr_t>(B)) & 15u) == 0;
  if (!aligned || M < 64) {
    bgemm_launch<float>(batch, M, N, K, alpha, A, lda, sA, B, ldb, sB, beta, C, ldc, sC, s);
    return;
  }
  for (int b0 = 0; b0 < batch; b0 += 65535) {
    const int nb = batch - b0 < 65535 ? batch - b0 : 65535;
    dim3 grid(ceil_div(N, 128), ceil_div(M, 128), nb);
    ves_count_launch();
    bgemm128_f32_kernel<<<grid, 256, 0, s>>>(M, N, K, alpha, A + b0 * sA, lda, sA, B + b0 * sB, ldb, sB, beta,
                                             C + b0 * sC, ldc, sC);
  }
}

// ----------------------------------------------------------------------------
// y[k] = A[k] (m x n) x[k]; one CTA per vesicle, one warp per row.
__global__ void bgemv_kernel(int m, int n, const double* __restrict__ A, const double* __restrict__ x,
                             long long xs, double* __restrict__ y, long long ys) {
  extern __shared__ double xsh[];
  const int k = blockIdx.x;
  for (int i = threadIdx.x; i < n; i += blockDim.x) xsh[i] = x[(long long)k * xs + i];
  __syncthreads();
  const int warp = threadIdx.x / 32, lane = threadIdx.x % 32, nw = blockDim.x / 32;
  const double* Ak = A + (long long)k * m * n;
  for (int r = warp; r < m; r += nw) {
    double s = 0.0;
    for (int c = lane; c < n; c += 32) s = fma(Ak[(long long)r * n + c], xsh[c], s);
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
    if (lane == 0) y[(long long)k * ys + r] = s;
  }
}

void launch_bgemv_f64(int nv, int m, int n, const double* A, const double* x, long long xs, double* y,
                      long long ys, cudaStream_t s) {
  if (nv <= 0) return;
  ves_count_launch();
  bgemv_kernel<<<nv, 256, (size_t)n * sizeof(double), s>>>(m, n, A, x, xs, y, ys);
}

// ----------------------------------------------------------------------------
// Blocked right-looking LU with partial pivoting, one CTA per matrix
// (the factorisation torch.linalg.lu_factor performs, tstep_biem.py:350).
// piv[j] = row exchanged with row j at step j (LAPACK ipiv, 0-based).
constexpr int LU_NB = 32;

template <typename T>
__global__ void __launch_bounds__(256) lu_factor_kernel(int n, T* __restrict__ A, int* __restrict__ piv,
                                                        VesDeviceStatus* st) {
  extern __shared__ __align__(16) unsigned char lu_sh[];
  T* sh = (T*)lu_sh;
  const int k = blockIdx.x;
  T* a = A + (long long)k * n * n;
  int* pv = piv + (long long)k * n;
  T* panel = sh;                 // [n][LU_NB]
  T* U12 = sh + n * LU_NB;       // [LU_NB][n]
  __shared__ double red_v[256];
  __shared__ int red_i[256];
  __shared__ int s_piv;
  const int tid = threadIdx.x, nt = blockDim.x;

  for (int p0 = 0; p0 < n; p0 += LU_NB) {
    const int nb = min(LU_NB, n - p0);
    const int rows = n - p0;
    for (int idx = tid; idx < rows * nb; idx += nt) {
      const int i = idx / nb, j = idx % nb;
      panel[i * LU_NB + j] = a[(long long)(p0 + i) * n + p0 + j];
    }
    __syncthreads();
    for (int j = 0; j < nb; ++j) {
      // pivot: first index of max |panel[i][j]|, i >= j
      double best = -1.0;
      int bi = n;
      for (int i = j + tid; i < rows; i += nt) {
        const double v = fabs((double)panel[i * LU_NB + j]);
        if (v > best) {
          best = v;
          bi = i;
        }
      }
      red_v[tid] = best;
      red_i[tid] = bi;
      __syncthreads();
      for (int w = nt / 2; w > 0; w >>= 1) {
        if (tid < w) {
          const double v2 = red_v[tid + w];
          const int i2 = red_i[tid + w];
          if (v2 > red_v[tid] || (v2 == red_v[tid] && i2 < red_i[tid])) {
            red_v[tid] = v2;
            red_i[tid] = i2;
          }
        }
        __syncthreads();
      }
      if (tid == 0) {
        s_piv = red_i[0];
        pv[p0 + j] = p0 + red_i[0];
        if (red_v[0] == 0.0) ves_set_error(st, VES_ERR_SINGULAR, 1, (long long)k * n + p0 + j);
      }
      __syncthreads();
      const int ip = s_piv;
      if (ip != j) {
        for (int jj = tid; jj < nb; jj += nt) {
          const T t = panel[j * LU_NB + jj];
          panel[j * LU_NB + jj] = panel[ip * LU_NB + jj];
          panel[ip * LU_NB + jj] = t;
        }
      }
      __syncthreads();
      const T d = panel[j * LU_NB + j];
      const T rcp = (d != T(0)) ? T(1) / d : T(0);
      for (int i = j + 1 + tid; i < rows; i += nt) panel[i * LU_NB + j] *= rcp;
      __syncthreads();
      const int rem = nb - j - 1;
      if (rem > 0) {
        for (int idx = tid; idx < (rows - j - 1) * rem; idx += nt) {
          const int i = j + 1 + idx / rem, jj = j + 1 + idx % rem;
          panel[i * LU_NB + jj] = fma(-panel[i * LU_NB + j], panel[j * LU_NB + jj], panel[i * LU_NB + jj]);
        }
      }
      __syncthreads();
    }
    // write the panel back
    for (int idx = tid; idx < rows * nb; idx += nt) {
      const int i = idx / nb, j = idx % nb;
      a[(long long)(p0 + i) * n + p0 + j] = panel[i * LU_NB + j];
    }
    // apply this panel's row exchanges to the columns left and right of it
    for (int j = 0; j < nb; ++j) {
      const int r1 = p0 + j, r2 = pv[p0 + j];
      if (r2 != r1) {
        for (int c = tid; c < n; c += nt) {
          if (c >= p0 && c < p0 + nb) continue;
          const T t = a[(long long)r1 * n + c];
          a[(long long)r1 * n + c] = a[(long long)r2 * n + c];
          a[(long long)r2 * n + c] = t;
        }
      }
      __syncthreads();
    }
    const int ncol = n - p0 - nb;
    if (ncol > 0) {
      // U12 = L11^{-1} A12 (unit lower triangular), one thread per column
      for (int c = tid; c < ncol; c += nt) {
        T col[LU_NB];
#pragma unroll
        for (int j = 0; j < LU_NB; ++j)
          if (j < nb) col[j] = a[(long long)(p0 + j) * n + p0 + nb + c];
#pragma unroll
        for (int j = 0; j < LU_NB; ++j) {
          if (j >= nb) break;
          const T v = col[j];
          for (int i = j + 1; i < nb; ++i) col[i] = fma(-panel[i * LU_NB + j], v, col[i]);
        }
#pragma unroll
        for (int j = 0; j < LU_NB; ++j)
          if (j < nb) {
            U12[j * n + c] = col[j];
            a[(long long)(p0 + j) * n + p0 + nb + c] = col[j];
          }
      }
      __syncthreads();
      // A22 -= L21 * U12
      const int m2 = rows - nb;
      for (long long idx = tid; idx < (long long)m2 * ncol; idx += nt) {
        const int i = (int)(idx / ncol), c = (int)(idx % ncol);
        T s = a[(long long)(p0 + nb + i) * n + p0 + nb + c];
        const T* l = panel + (nb + i) * LU_NB;
#pragma unroll 8
        for (int j = 0; j < nb; ++j) s = fma(-l[j], U12[j * n + c], s);
        a[(long long)(p0 + nb + i) * n + p0 + nb + c] = s;
      }
    }
    __syncthreads();
  }
}

template <typename T>
static int lu_factor_t(ves_ctx* c, int nv, int n, T* A, int* piv, cudaStream_t s) {
  if (nv <= 0) return VES_OK;
  const size_t sh = (size_t)(n * LU_NB + LU_NB * n) * sizeof(T);
  if (sh > 220 * 1024) {
    ves_record_error(VES_ERR_SHAPE, "lu_factor: n=%d too large", n);
    return VES_ERR_SHAPE;
  }
  if (sh > 32 * 1024) {  // dynamic + static shared memory must fit the opt-in limit
    int rc = ves_cuda_status(
        cudaFuncSetAttribute(lu_factor_kernel<T>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sh),
        "lu_factor smem attribute");
    if (rc) return rc;
  }
  ves_count_launch();
  lu_factor_kernel<T><<<nv, 256, sh, s>>>(n, A, piv, c->status);
  return ves_launch_check("lu_factor");
}

int launch_lu_factor(ves_ctx* c, int nv, int n, double* A, int* piv, cudaStream_t s) {
  return lu_factor_t<double>(c, nv, n, A, piv, s);
}

int launch_lu_factor_f32(ves_ctx* c, int nv, int n, float* A, int* piv, cudaStream_t s) {
  return lu_factor_t<float>(c, nv, n, A, piv, s);
}

// x = LU^{-1} P b per vesicle.  Blocks of 32 rows: the off-diagonal part is a
// warp-parallel GEMV, the 32x32 diagonal block is solved by one warp.
template <typename T>
__global__ void __launch_bounds__(256) lu_solve_kernel(int n, const T* __restrict__ LU,
                                                       const int* __restrict__ piv,
                                                       const double* __restrict__ b, double* __restrict__ x) {
  extern __shared__ double xs[];
  const int k = blockIdx.x;
  const T* a = LU + (long long)k * n * n;
  const int* pv = piv + (long long)k * n;
  const int tid = threadIdx.x, warp = tid / 32, lane = tid % 32, nw = blockDim.x / 32;
  for (int i = tid; i < n; i += blockDim.x) xs[i] = b[(long long)k * n + i];
  __syncthreads();
  if (tid == 0) {
    for (int j = 0; j < n; ++j) {
      const int p = pv[j];
      if (p != j) {
        const double t = xs[j];
        xs[j] = xs[p];
        xs[p] = t;
      }
    }
  }
  __syncthreads();
  // forward: unit lower
  for (int r0 = 0; r0 < n; r0 += 32) {
    const int nr = min(32, n - r0);
    for (int r = warp; r < nr; r += nw) {
      double s = 0.0;
      for (int c = lane; c < r0; c += 32) s = fma((double)a[(long long)(r0 + r) * n + c], xs[c], s);
#pragma unroll
      for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
      if (lane == 0) xs[r0 + r] -= s;
    }
    __syncthreads();
    if (warp == 0) {
      double v = (lane < nr) ? xs[r0 + lane] : 0.0;
      for (int j = 0; j < nr; ++j) {
        const double xj = __shfl_sync(0xffffffffu, v, j);
        if (lane > j && lane < nr) v = fma(-(double)a[(long long)(r0 + lane) * n + r0 + j], xj, v);
      }
      if (lane < nr) xs[r0 + lane] = v;
    }
    __syncthreads();
  }
  // backward: upper
  for (int r1 = n; r1 > 0; r1 -= 32) {
    const int r0 = max(0, r1 - 32), nr = r1 - r0;
    for (int r = warp; r < nr; r += nw) {
      double s = 0.0;
      for (int c = r1 + lane; c < n; c += 32) s = fma((double)a[(long long)(r0 + r) * n + c], xs[c], s);
#pragma unroll
      for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
      if (lane == 0) xs[r0 + r] -= s;
    }
    __syncthreads();
    if (warp == 0) {
      double v = (lane < nr) ? xs[r0 + lane] : 0.0;
      for (int j = nr - 1; j >= 0; --j) {
        double vj = __shfl_sync(0xffffffffu, v, j);
        if (lane == j) {
          v = v / (double)a[(long long)(r0 + j) * n + r0 + j];
        }
        vj = __shfl_sync(0xffffffffu, v, j);
        if (lane < j) v = fma(-(double)a[(long long)(r0 + lane) * n + r0 + j], vj, v);
      }
      if (lane < nr) xs[r0 + lane] = v;
    }
    __syncthreads();
  }
  for (int i = tid; i < n; i += blockDim.x) x[(long long)k * n + i] = xs[i];
}

void launch_lu_solve(int nv, int n, const double* LU, const int* piv, const double* b, double* x,
                     cudaStream_t s) {
  if (nv <= 0) return;
  ves_count_launch();
  lu_solve_kernel<double><<<nv, 256, (size_t)n * sizeof(double), s>>>(n, LU, piv, b, x);
}

// the same solve with an FP32 factorisation (FP64 right-hand side, FP64 sums)
void launch_lu_solve_f32(int nv, int n, const float* LU, const int* piv, const double* b, double* x,
                         cudaStream_t s) {
  if (nv <= 0) return;
  ves_count_launch();
  lu_solve_kernel<float><<<nv, 256, (size_t)n * sizeof(double), s>>>(n, LU, piv, b, x);
}

// ----------------------------------------------------------------------------
// Deterministic dot product: fixed number of blocks, fixed reduction order.
constexpr int DOT_BLOCKS = 512;
int dot_partial_blocks() { return DOT_BLOCKS; }

__global__ void __launch_bounds__(256) dot_partials_kernel(long long n, const double* __restrict__ a,
                                                           const double* __restrict__ b,
                                                           double* __restrict__ partials) {
  __shared__ double red[256];
  double s = 0.0;
  for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x)
    s = fma(a[i], b[i], s);
  red[threadIdx.x] = s;
  __syncthreads();
  for (int w = 128; w > 0; w >>= 1) {
    if (threadIdx.x < w) red[threadIdx.x] += red[threadIdx.x + w];
    __syncthreads();
  }
  if (threadIdx.x == 0) partials[blockIdx.x] = red[0];
}

void launch_dot_partials(long long n, const double* a, const double* b, double* partials, cudaStream_t s) {
  ves_count_launch();
  dot_partials_kernel<<<DOT_BLOCKS, 256, 0, s>>>(n, a, b, partials);
}
