// k_mlp.cu -- the small MLP of the learned lambda schedule: forward pass,
// backward pass and Adam update, hand-written for one thread block.
//
// Network: x[F] -> tanh(W1 x + b1)[128] -> tanh(W2 h1 + b2)[128] -> W3 h2 + b3
// [1], over a batch of up to QM_B rows (lambda windows).  The three layer
// products run on the tensor cores with mma.sync m16n8k16 (BF16 operands,
// FP32 accumulation); weights are held in BF16 for the products and as FP32
// master copies (with the Adam moments) for the update.  Sizes are padded:
// F to QM_F = 16 inputs, the output to QM_O = 16 columns (column 0 is the
// prediction).  One launch runs `iters` full-batch training steps in a fixed
// order, so training is deterministic.  The C-ABI entry points at the end
// (qgpu_mlp_*) take host arrays.
#include <cuda_bf16.h>

#include "qgpu_internal.cuh"

#define QM_B 64      // batch rows (windows)
#define QM_F 16      // padded inputs
#define QM_H 128     // hidden width
#define QM_O 16      // padded outputs (column 0 used)
#define QM_THREADS 256

// parameter block layout (floats): W1[H][F] b1[H] W2[H][H] b2[H] W3[O][H] b3[O]
#define QM_NW1 (QM_H * QM_F)
#define QM_NW2 (QM_H * QM_H)
#define QM_NW3 (QM_O * QM_H)
#define QM_NP (QM_NW1 + QM_H + QM_NW2 + QM_H + QM_NW3 + QM_O)

struct MlpShared {
    __nv_bfloat16 w1[QM_H][QM_F], w2[QM_H][QM_H], w3[QM_O][QM_H];
    __nv_bfloat16 x[QM_B][QM_F], a1[QM_B][QM_H], a2[QM_B][QM_H];   // layer inputs (BF16)
    float h1[QM_B][QM_H], h2[QM_B][QM_H];                            // tanh outputs (FP32)
    float sc[QM_B][QM_H];                                            // backward scratch
    float y[QM_B][QM_O];
    __nv_bfloat16 g3[QM_B][QM_O], g2[QM_B][QM_H], g1[QM_B][QM_H];   // dL/d(pre-activation), BF16
    float loss[QM_THREADS / 32];
};

// D = A B + D for one 16x8x16 tile; a[4], b[2] are packed BF16 pairs
__device__ __forceinline__ void mma_bf16(float (&d)[4], const unsigned (&a)[4], const unsigned (&b)[2]) {
    asm volatile(
        "mma.sync.aligned.m16n8k16.row.col.f32.bf16.bf16.f32 {%0,%1,%2,%3}, {%4,%5,%6,%7}, {%8,%9}, "
        "{%0,%1,%2,%3};\n"
        : "+f"(d[0]), "+f"(d[1]), "+f"(d[2]), "+f"(d[3])
        : "r"(a[0]), "r"(a[1]), "r"(a[2]), "r"(a[3]), "r"(b[0]), "r"(b[1]));
}
__device__ __forceinline__ unsigned pack2(__nv_bfloat16 lo, __nv_bfloat16 hi) {
    return (unsigned)__bfloat16_as_ushort(lo) | ((unsigned)__bfloat16_as_ushort(hi) << 16);
}

// C[M][N] (FP32, row-major, ldc) = sum_k A(m, k) B(k, n) over K, for M, N, K
// multiples of 16, 8, 16; A and B are element functions (BF16).  Tiles are
// spread over the block's warps.  Fragment layout of m16n8k16 (PTX ISA):
// lane = 4 g + t; A regs (g, 2t..2t+1), (g+8, 2t..), (g, 2t+8..), (g+8, 2t+8..);
// B regs (k = 2t..2t+1, n = g), (k = 2t+8.., n = g); C (g, 2t..), (g+8, 2t..).
template <typename FA, typename FB>
__device__ void gemm_tiles(int M, int N, int K, FA A, FB B, float *C, int ldc) {
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31, g = lane >> 2, t = lane & 3;
    const int tn = N / 8, ntile = (M / 16) * tn;
    for (int tile = warp; tile < ntile; tile += blockDim.x >> 5) {
        const int m0 = (tile / tn) * 16, n0 = (tile % tn) * 8;
        float d[4] = {0.f, 0.f, 0.f, 0.f};
        for (int k0 = 0; k0 < K; k0 += 16) {
            unsigned a[4], b[2];
            a[0] = pack2(A(m0 + g, k0 + 2 * t), A(m0 + g, k0 + 2 * t + 1));
            a[1] = pack2(A(m0 + g + 8, k0 + 2 * t), A(m0 + g + 8, k0 + 2 * t + 1));
            a[2] = pack2(A(m0 + g, k0 + 2 * t + 8), A(m0 + g, k0 + 2 * t + 9));
            a[3] = pack2(A(m0 + g + 8, k0 + 2 * t + 8), A(m0 + g + 8, k0 + 2 * t + 9));
            b[0] = pack2(B(k0 + 2 * t, n0 + g), B(k0 + 2 * t + 1, n0 + g));
            b[1] = pack2(B(k0 + 2 * t + 8, n0 + g), B(k0 + 2 * t + 9, n0 + g));
            mma_bf16(d, a, b);
        }
        C[(m0 + g) * ldc + n0 + 2 * t] = d[0];
        C[(m0 + g) * ldc + n0 + 2 * t + 1] = d[1];
        C[(m0 + g + 8) * ldc + n0 + 2 * t] = d[2];
        C[(m0 + g + 8) * ldc + n0 + 2 * t + 1] = d[3];
    }
}

__device__ void load_weights(MlpShared &sh, const float *P) {
    const float *W1 = P, *W2 = P + QM_NW1 + QM_H, *W3 = W2 + QM_NW2 + QM_H;
    for (int i = threadIdx.x; i < QM_NW1; i += blockDim.x) sh.w1[i / QM_F][i % QM_F] = __float2bfloat16(W1[i]);
    for (int i = threadIdx.x; i < QM_NW2; i += blockDim.x) sh.w2[i / QM_H][i % QM_H] = __float2bfloat16(W2[i]);
    for (int i = threadIdx.x; i < QM_NW3; i += blockDim.x) sh.w3[i / QM_H][i % QM_H] = __float2bfloat16(W3[i]);
}

// forward over rows [0, QM_B): h1, h2 (tanh), y (linear); rows >= n are zero input
__device__ void forward(MlpShared &sh, const float *P, const float *X, int n) {
    const float *b1 = P + QM_NW1, *b2 = b1 + QM_H + QM_NW2, *b3 = b2 + QM_H + QM_NW3;
    for (int i = threadIdx.x; i < QM_B * QM_F; i += blockDim.x) {
        const int r = i / QM_F, c = i % QM_F;
        sh.x[r][c] = __float2bfloat16(r < n ? X[r * QM_F + c] : 0.f);
    }
    __syncthreads();
    gemm_tiles(QM_B, QM_H, QM_F, [&](int m, int k) { return sh.x[m][k]; },
               [&](int k, int nn) { return sh.w1[nn][k]; }, &sh.h1[0][0], QM_H);
    __syncthreads();
    for (int i = threadIdx.x; i < QM_B * QM_H; i += blockDim.x) {
        const int r = i / QM_H, c = i % QM_H;
        const float v = tanhf(sh.h1[r][c] + b1[c]);
        sh.h1[r][c] = v;
        sh.a1[r][c] = __float2bfloat16(v);
    }
    __syncthreads();
    gemm_tiles(QM_B, QM_H, QM_H, [&](int m, int k) { return sh.a1[m][k]; },
               [&](int k, int nn) { return sh.w2[nn][k]; }, &sh.h2[0][0], QM_H);
    __syncthreads();
    for (int i = threadIdx.x; i < QM_B * QM_H; i += blockDim.x) {
        const int r = i / QM_H, c = i % QM_H;
        const float v = tanhf(sh.h2[r][c] + b2[c]);
        sh.h2[r][c] = v;
        sh.a2[r][c] = __float2bfloat16(v);
    }
    __syncthreads();
    gemm_tiles(QM_B, QM_O, QM_H, [&](int m, int k) { return sh.a2[m][k]; },
               [&](int k, int nn) { return sh.w3[nn][k]; }, &sh.y[0][0], QM_O);
    __syncthreads();
    for (int i = threadIdx.x; i < QM_B * QM_O; i += blockDim.x) sh.y[i / QM_O][i % QM_O] += b3[i % QM_O];
    __syncthreads();
}

// Inference: out[n] = prediction of each row.
__global__ void __launch_bounds__(QM_THREADS) k_mlp_forward(const float *P, const float *X, int n, float *out) {
    extern __shared__ __align__(16) unsigned char smem[];
    MlpShared &sh = *reinterpret_cast<MlpShared *>(smem);
    load_weights(sh, P);
    forward(sh, P, X, n);
    for (int r = threadIdx.x; r < n; r += blockDim.x) out[r] = sh.y[r][0];
}

// iters full-batch steps of Adam on the loss 1/n sum_r (y_r - target_r)^2.
// P: FP32 parameters (updated in place); Mo, Vo: Adam moments; G: gradient
// buffer (QM_NP floats, the last step's gradient is left there); loss_out[iters]
// (may be null) the loss before each update.  step0: Adam steps already taken.
__global__ void __launch_bounds__(QM_THREADS) k_mlp_train(float *P, float *Mo, float *Vo, float *G, const float *X,
                                                         const float *Ytgt, int n, int iters, float lr, int step0,
                                                         float *loss_out) {
    extern __shared__ __align__(16) unsigned char smem[];
    MlpShared &sh = *reinterpret_cast<MlpShared *>(smem);
    float *gW1 = G, *gb1 = G + QM_NW1, *gW2 = gb1 + QM_H, *gb2 = gW2 + QM_NW2, *gW3 = gb2 + QM_H, *gb3 = gW3 + QM_NW3;
    const float inv_n = 1.f / (float)n;
    for (int it = 0; it < iters; ++it) {
        load_weights(sh, P);
        __syncthreads();
        forward(sh, P, X, n);
        // output gradient dL/dy = 2 (y - t)/n (rows < n, column 0), loss
        float lsum = 0.f;
        for (int i = threadIdx.x; i < QM_B * QM_O; i += blockDim.x) {
            const int r = i / QM_O, c = i % QM_O;
            float gr = 0.f;
            if (r < n && c == 0) {
                const float e = sh.y[r][0] - Ytgt[r];
                lsum += e * e;
                gr = 2.f * e * inv_n;
            }
            sh.g3[r][c] = __float2bfloat16(gr);
            sh.y[r][c] = gr;   // FP32 copy of the output gradient
        }
        for (int o = 16; o > 0; o >>= 1) lsum += __shfl_xor_sync(0xffffffffu, lsum, o);
        if ((threadIdx.x & 31) == 0) sh.loss[threadIdx.x >> 5] = lsum;
        __syncthreads();
        if (threadIdx.x == 0 && loss_out) {
            float s = 0.f;
            for (int w = 0; w < QM_THREADS / 32; ++w) s += sh.loss[w];
            loss_out[it] = s * inv_n;
        }
        // layer 3: gW3[o][k] = sum_r g3[r][o] a2[r][k]; gb3 = sum_r g3; d a2 = g3 W3
        gemm_tiles(QM_O, QM_H, QM_B, [&](int m, int kk) { return sh.g3[kk][m]; },
                   [&](int kk, int nn) { return sh.a2[kk][nn]; }, gW3, QM_H);
        for (int c = threadIdx.x; c < QM_O; c += blockDim.x) {
            float s = 0.f;
            for (int r = 0; r < QM_B; ++r) s += sh.y[r][c];
            gb3[c] = s;
        }
        gemm_tiles(QM_B, QM_H, QM_O, [&](int m, int kk) { return sh.g3[m][kk]; },
                   [&](int kk, int nn) { return sh.w3[kk][nn]; }, &sh.sc[0][0], QM_H);
        __syncthreads();
        // through tanh of layer 2: g2 = d a2 (1 - h2^2), d a2 in the scratch
        for (int i = threadIdx.x; i < QM_B * QM_H; i += blockDim.x) {
            const int r = i / QM_H, c = i % QM_H;
            const float v = sh.sc[r][c] * (1.f - sh.h2[r][c] * sh.h2[r][c]);
            sh.g2[r][c] = __float2bfloat16(v);
            sh.h2[r][c] = v;   // FP32 copy for the bias gradient
        }
        __syncthreads();
        gemm_tiles(QM_H, QM_H, QM_B, [&](int m, int kk) { return sh.g2[kk][m]; },
                   [&](int kk, int nn) { return sh.a1[kk][nn]; }, gW2, QM_H);
        for (int c = threadIdx.x; c < QM_H; c += blockDim.x) {
            float s = 0.f;
            for (int r = 0; r < QM_B; ++r) s += sh.h2[r][c];
            gb2[c] = s;
        }
        gemm_tiles(QM_B, QM_H, QM_H, [&](int m, int kk) { return sh.g2[m][kk]; },
                   [&](int kk, int nn) { return sh.w2[kk][nn]; }, &sh.sc[0][0], QM_H);
        __syncthreads();
        // through tanh of layer 1: g1 = d a1 (1 - h1^2)
        for (int i = threadIdx.x; i < QM_B * QM_H; i += blockDim.x) {
            const int r = i / QM_H, c = i % QM_H;
            const float v = sh.sc[r][c] * (1.f - sh.h1[r][c] * sh.h1[r][c]);
            sh.g1[r][c] = __float2bfloat16(v);
            sh.h2[r][c] = v;
        }
        __syncthreads();
        gemm_tiles(QM_H, QM_F, QM_B, [&](int m, int kk) { return sh.g1[kk][m]; },
                   [&](int kk, int nn) { return sh.x[kk][nn]; }, gW1, QM_F);
        for (int c = threadIdx.x; c < QM_H; c += blockDim.x) {
            float s = 0.f;
            for (int r = 0; r < QM_B; ++r) s += sh.h2[r][c];
            gb1[c] = s;
        }
        __syncthreads();
        __threadfence_block();
        // Adam (beta1 0.9, beta2 0.999, eps 1e-8), bias-corrected
        const int st = step0 + it + 1;
        const float c1 = 1.f - powf(0.9f, (float)st), c2 = 1.f - powf(0.999f, (float)st);
        for (int i = threadIdx.x; i < QM_NP; i += blockDim.x) {
            const float gi = G[i];
            const float m = 0.9f * Mo[i] + 0.1f * gi, v = 0.999f * Vo[i] + 0.001f * gi * gi;
            Mo[i] = m; Vo[i] = v;
            P[i] -= lr * (m / c1) / (sqrtf(v / c2) + 1e-8f);
        }
        __syncthreads();
        __threadfence_block();
    }
}

// ------------------------------------------------------------------ C-ABI
// Host arrays in and out; device buffers live for the call only.
namespace {
struct DevBuf {
    void *p = nullptr;
    ~DevBuf() { if (p) cudaFree(p); }
};
int mlp_prepare() {
    if (cudaFuncSetAttribute(k_mlp_forward, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sizeof(MlpShared)) !=
            cudaSuccess ||
        cudaFuncSetAttribute(k_mlp_train, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sizeof(MlpShared)) !=
            cudaSuccess)
        return qgpu_fail(QGPU_E_CUDA, "MLP kernels: %s", cudaGetErrorString(cudaGetLastError()));
    return 0;
}
int up(DevBuf &b, const void *src, size_t bytes) {
    if (cudaMalloc(&b.p, bytes ? bytes : 4) != cudaSuccess) return qgpu_fail(QGPU_E_CUDA, "MLP: cudaMalloc failed");
    if (src && bytes && cudaMemcpy(b.p, src, bytes, cudaMemcpyHostToDevice) != cudaSuccess)
        return qgpu_fail(QGPU_E_CUDA, "MLP: copy failed");
    if (!src && bytes && cudaMemset(b.p, 0, bytes) != cudaSuccess) return qgpu_fail(QGPU_E_CUDA, "MLP: memset failed");
    return 0;
}
int down(void *dst, const DevBuf &b, size_t bytes) {
    if (dst && cudaMemcpy(dst, b.p, bytes, cudaMemcpyDeviceToHost) != cudaSuccess)
        return qgpu_fail(QGPU_E_CUDA, "MLP: copy back failed: %s", cudaGetErrorString(cudaGetLastError()));
    return 0;
}
}  // namespace

extern "C" int qgpu_mlp_nparams(void) { return QM_NP; }

extern "C" int qgpu_mlp_predict(const float *params, const float *X, int32_t n, float *out) {
    if (!params || !X || !out || n < 1 || n > QM_B) return qgpu_fail(QGPU_E_INVALID, "qgpu_mlp_predict: bad arguments");
    if (int rc = mlp_prepare()) return rc;
    DevBuf P, Xd, O;
    int rc;
    if ((rc = up(P, params, QM_NP * sizeof(float))) || (rc = up(Xd, X, (size_t)n * QM_F * sizeof(float))) ||
        (rc = up(O, nullptr, (size_t)n * sizeof(float))))
        return rc;
    k_mlp_forward<<<1, QM_THREADS, sizeof(MlpShared)>>>((const float *)P.p, (const float *)Xd.p, n, (float *)O.p);
    return down(out, O, (size_t)n * sizeof(float));
}

extern "C" int qgpu_mlp_train(float *params, float *adam_m, float *adam_v, const float *X, const float *Y, int32_t n,
                              int32_t iters, float lr, int32_t step0, float *loss_out, float *grad_out) {
    if (!params || !adam_m || !adam_v || !X || !Y || n < 1 || n > QM_B || iters < 1 || step0 < 0)
        return qgpu_fail(QGPU_E_INVALID, "qgpu_mlp_train: bad arguments");
    if (int rc = mlp_prepare()) return rc;
    DevBuf P, M, V, G, Xd, Yd, L;
    const size_t np = QM_NP * sizeof(float);
    int rc;
    if ((rc = up(P, params, np)) || (rc = up(M, adam_m, np)) || (rc = up(V, adam_v, np)) || (rc = up(G, nullptr, np)) ||
        (rc = up(Xd, X, (size_t)n * QM_F * sizeof(float))) || (rc = up(Yd, Y, (size_t)n * sizeof(float))) ||
        (rc = up(L, nullptr, (size_t)iters * sizeof(float))))
        return rc;
    k_mlp_train<<<1, QM_THREADS, sizeof(MlpShared)>>>((float *)P.p, (float *)M.p, (float *)V.p, (float *)G.p,
                                                      (const float *)Xd.p, (const float *)Yd.p, n, iters, lr, step0,
                                                      (float *)L.p);
    if ((rc = down(params, P, np)) || (rc = down(adam_m, M, np)) || (rc = down(adam_v, V, np)) ||
        (rc = down(loss_out, L, (size_t)iters * sizeof(float))) || (rc = down(grad_out, G, np)))
        return rc;
    return 0;
}
