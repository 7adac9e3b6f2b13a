// kernels_gemm.cu -- batched FP32 GEMM  C[b][m][n] = sum_k A[b][m][k] * B[n][k]
// (both operands K-contiguous; B shared by the batch).  Used for the whitening /
// drift-correction product (X <- (M @ Wrot) @ X, Kilosort io.py:784-790, done on
// time-major rows as Z = Y (M Wrot)^T) and for the projection onto the templates
// (B = Wall3 . Bpc, Kilosort template_matching.py:146).
//
// 128x128 output tile per CTA, 256 threads with an 8x8 register tile each, K stepped by 8
// through double-buffered shared memory.
#include "lss_kernels.cuh"

namespace lss {

constexpr int kTM = 128, kTN = 128, kTK = 8;

__global__ void __launch_bounds__(256)
sgemm_nt_kernel(const float* __restrict__ A, int64_t lda, int64_t strideA, const float* __restrict__ B,
                int64_t ldb, float* __restrict__ Cm, int64_t ldc, int64_t strideC, int M, int N, int K) {
    __shared__ __align__(16) float As[2][kTK][kTM];
    __shared__ __align__(16) float Bs[2][kTK][kTN];
    const int b = blockIdx.z;
    const float* Ab = A + (int64_t)b * strideA;
    float* Cb = Cm + (int64_t)b * strideC;
    const int m0 = blockIdx.y * kTM, n0 = blockIdx.x * kTN;
    const int tid = threadIdx.x;
    const int tx = tid & 15, ty = tid >> 4;
    // loader mapping: 256 threads x 4 elements = 128 rows x 8 k
    const int lrow = tid >> 1, lk = (tid & 1) * 4;

    float ra[4], rb[4];
    auto load_regs = [&](int k0) {
        const int am = m0 + lrow, bn = n0 + lrow;
#pragma unroll
        for (int i = 0; i < 4; ++i) {
            const int k = k0 + lk + i;
            ra[i] = (am < M && k < K) ? __ldg(Ab + (int64_t)am * lda + k) : 0.f;
            rb[i] = (bn < N && k < K) ? __ldg(B + (int64_t)bn * ldb + k) : 0.f;
        }
    };
    auto store_smem = [&](int buf) {
#pragma unroll
        for (int i = 0; i < 4; ++i) {
            As[buf][lk + i][lrow] = ra[i];
            Bs[buf][lk + i][lrow] = rb[i];
        }
    };

    float acc[8][8];
#pragma unroll
    for (int i = 0; i < 8; ++i)
#pragma unroll
        for (int j = 0; j < 8; ++j) acc[i][j] = 0.f;

    const int nk = (K + kTK - 1) / kTK;
    load_regs(0);
    store_smem(0);
    __syncthreads();
    for (int kt = 0; kt < nk; ++kt) {
        const int buf = kt & 1;
        if (kt + 1 < nk) load_regs((kt + 1) * kTK);
#pragma unroll
        for (int kk = 0; kk < kTK; ++kk) {
            float a[8], bv[8];
            const float4 a0 = *reinterpret_cast<const float4*>(&As[buf][kk][ty * 4]);
            const float4 a1 = *reinterpret_cast<const float4*>(&As[buf][kk][64 + ty * 4]);
            const float4 b0 = *reinterpret_cast<const float4*>(&Bs[buf][kk][tx * 4]);
            const float4 b1 = *reinterpret_cast<const float4*>(&Bs[buf][kk][64 + tx * 4]);
            a[0] = a0.x; a[1] = a0.y; a[2] = a0.z; a[3] = a0.w;
            a[4] = a1.x; a[5] = a1.y; a[6] = a1.z; a[7] = a1.w;
            bv[0] = b0.x; bv[1] = b0.y; bv[2] = b0.z; bv[3] = b0.w;
            bv[4] = b1.x; bv[5] = b1.y; bv[6] = b1.z; bv[7] = b1.w;
#pragma unroll
            for (int i = 0; i < 8; ++i)
#pragma unroll
                for (int j = 0; j < 8; ++j) acc[i][j] = fmaf(a[i], bv[j], acc[i][j]);
        }
        if (kt + 1 < nk) store_smem(buf ^ 1);
        __syncthreads();
    }
    // rows: ty*4 + {0..3} and 64 + ty*4 + {0..3}; cols likewise with tx
#pragma unroll
    for (int i = 0; i < 8; ++i) {
        const int m = m0 + (i < 4 ? ty * 4 + i : 64 + ty * 4 + (i - 4));
        if (m >= M) continue;
#pragma unroll
        for (int j = 0; j < 8; ++j) {
            const int n = n0 + (j < 4 ? tx * 4 + j : 64 + tx * 4 + (j - 4));
            if (n < N) Cb[(int64_t)m * ldc + n] = acc[i][j];
        }
    }
}

void launch_sgemm_nt(const float* A, int64_t lda, int64_t strideA, const float* B, int64_t ldb, float* Cm,
                     int64_t ldc, int64_t strideC, int M, int N, int K, int nb, cudaStream_t s) {
    dim3 grid((N + kTN - 1) / kTN, (M + kTM - 1) / kTM, nb);
    sgemm_nt_kernel<<<grid, 256, 0, s>>>(A, lda, strideA, B, ldb, Cm, ldc, strideC, M, N, K);
}

}  // namespace lss
