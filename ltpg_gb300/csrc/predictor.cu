// predictor.cu — contention predictor: which key-hash buckets to stage.
//
// Input per bucket: log1p of its registration counts in the last 4 batches
// (counted by the tuned execute kernels).  Model: MLP 4 -> 64 -> 64 -> 1 with
// ReLU, BF16 weights and activations, FP32 accumulation; the output predicts
// log1p of the bucket's count in the next batch.  After every batch:
//   roll      the batch's counts enter a 5-batch ring and the counters reset;
//   train     one Adam step on 4,096 buckets (a rotating 1/16 of them): the
//             features are batches t-5..t-2, the label batch t-1 (the "previous
//             batch's registration contention");
//   infer     all 65,536 buckets from batches t-4..t-1;
//   select    the top-k scores become the staged set (k = staging groups).
// Six kernels per batch: roll (+ ring advance), training forward, fused
// backward (+ loss), Adam (+ BF16 copies), inference forward, select (+ step
// counters).
// The forward pass runs on the tensor cores (mma.sync m16n8k16, BF16 inputs,
// FP32 accumulators); backward and Adam are FP32.  The predictor only picks
// the staged set, which changes speed, never a commit decision.
#include <cuda_bf16.h>

#include <cstring>
#include <vector>

#include "stage.cuh"

namespace ltpg {

constexpr int PH = 64;            // hidden width
constexpr int PF = 4;             // features (batches of history)
constexpr int P_RING = 5;         // count ring: 4 feature batches + 1 label batch
constexpr int P_TRAIN = 4096;     // samples per training step
constexpr int P_W1 = 0, P_B1 = P_W1 + PH * PF, P_W2 = P_B1 + PH, P_B2 = P_W2 + PH * PH, P_W3 = P_B2 + PH,
              P_B3 = P_W3 + PH, P_NPARAM = P_B3 + 1;  // packed FP32 parameter layout

struct PredDev {
    float *param, *m, *v, *grad;          // P_NPARAM each
    __nv_bfloat16 *w1b, *w2b;             // BF16 copies: w1b [64][16] (K padded), w2b [64][64]
    uint32_t *ring;                       // P_RING x buckets
    float *scores;                        // buckets
    float *act;                           // training activations: X [S][4], H1 [S][64], H2 [S][64], Y [S], T [S]
    uint32_t *state;                      // [0] ring position, [1] step, [2] batches seen, [3] blocks done
    float *loss;                          // [0] last training loss, [1] its running sum over sample tiles
};

__device__ __forceinline__ uint32_t pack_bf16(float lo, float hi) {
    const __nv_bfloat162 v = __floats2bfloat162_rn(lo, hi);
    return *reinterpret_cast<const uint32_t *>(&v);
}

__device__ __forceinline__ void mma_bf16(float *d, const uint32_t *a, const uint32_t *b) {
    asm volatile(
        "mma.sync.aligned.m16n8k16.row.col.f32.bf16.bf16.f32 {%0,%1,%2,%3}, {%4,%5,%6,%7}, {%8,%9}, "
        "{%0,%1,%2,%3};"
        : "+f"(d[0]), "+f"(d[1]), "+f"(d[2]), "+f"(d[3])
        : "r"(a[0]), "r"(a[1]), "r"(a[2]), "r"(a[3]), "r"(b[0]), "r"(b[1]));
}

// Features of bucket b: log1p of its counts in the 4 ring slots ending at
// `newest` (oldest first).
__device__ __forceinline__ void features(const uint32_t *ring, uint32_t newest, uint32_t b, float *x) {
#pragma unroll
    for (int f = 0; f < PF; ++f) {
        const uint32_t slot = (newest + P_RING - (PF - 1 - f)) % P_RING;
        x[f] = log1pf((float)ring[slot * STAGE_BUCKETS + b]);
    }
}

// ---- forward on tensor cores ----------------------------------------------------
// A warp runs 16 samples at a time.  Layer 1: [16 x 16] (4 features, zero
// padded) x W1^T -> 8 n-tiles of 8; the FP32 accumulators of tiles 2kb and
// 2kb+1, after bias + ReLU + BF16 rounding, are exactly the A fragment of
// k-block kb of layer 2 (16 x 64 x 64, 32 mma).  Layer 3 is a dot product
// reduced over the 4 lanes that share a row.
// mode 0: inference over `n` buckets (x from the ring, newest = slot t-1),
//         writes scores.  mode 1: training samples (x from slots t-5..t-2),
//         also stores X, H1, H2, Y, T for the backward pass.
// mode 2: x given in `xin` [n][4] (tests), writes y.  mode 3: x given in `xin`,
//         stores X, H1, H2, Y like mode 1 (the gradient test sets T).
__global__ void __launch_bounds__(256) pred_forward(PredDev p, uint32_t n, int mode, const float *__restrict__ xin,
                                                    float *__restrict__ yout) {
    __shared__ __align__(16) __nv_bfloat16 w1s[PH * 16];
    __shared__ __align__(16) __nv_bfloat16 w2s[PH * PH];
    __shared__ float b1s[PH], b2s[PH], w3s[PH];
    __shared__ float b3s;
    for (int i = threadIdx.x; i < PH * 16; i += blockDim.x) w1s[i] = p.w1b[i];
    for (int i = threadIdx.x; i < PH * PH; i += blockDim.x) w2s[i] = p.w2b[i];
    for (int i = threadIdx.x; i < PH; i += blockDim.x) {
        b1s[i] = p.param[P_B1 + i];
        b2s[i] = p.param[P_B2 + i];
        w3s[i] = p.param[P_W3 + i];
    }
    if (threadIdx.x == 0) b3s = p.param[P_B3];
    __syncthreads();
    const uint32_t lane = threadIdx.x & 31, g = lane >> 2, q = lane & 3;
    const uint32_t pos = p.state[0], step = p.state[1];
    const uint32_t newest = (pos + P_RING - 1) % P_RING;  // slot of batch t-1
    const uint32_t warp = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const uint32_t n_warps = (gridDim.x * blockDim.x) >> 5;
    for (uint32_t s0 = warp * 16; s0 < n; s0 += n_warps * 16) {
        // sample ids of rows g and g + 8
        uint32_t sid[2] = {s0 + g, s0 + g + 8};
        float xr[2][PF], tr[2] = {0.f, 0.f};
#pragma unroll
        for (int h = 0; h < 2; ++h) {
            const uint32_t s = sid[h];
#pragma unroll
            for (int f = 0; f < PF; ++f) xr[h][f] = 0.f;
            if (s >= n) continue;
            if (mode == 2 || mode == 3) {
#pragma unroll
                for (int f = 0; f < PF; ++f) xr[h][f] = xin[s * PF + f];
            } else if (mode == 1) {
                const uint32_t b = (s * 16u + (step & 15u)) & (STAGE_BUCKETS - 1u);  // rotating 1/16 of buckets
                features(p.ring, (newest + P_RING - 1) % P_RING, b, xr[h]);
                tr[h] = log1pf((float)p.ring[newest * STAGE_BUCKETS + b]);
            } else {
                features(p.ring, newest, s, xr[h]);
            }
        }
        // A fragment of layer 1: features are k = 0..3 (lanes q = 0, 1)
        uint32_t a1[4];
        a1[0] = q == 0 ? pack_bf16(xr[0][0], xr[0][1]) : q == 1 ? pack_bf16(xr[0][2], xr[0][3]) : 0u;
        a1[1] = q == 0 ? pack_bf16(xr[1][0], xr[1][1]) : q == 1 ? pack_bf16(xr[1][2], xr[1][3]) : 0u;
        a1[2] = 0u;
        a1[3] = 0u;
        float h1[8][4];
#pragma unroll
        for (int nt = 0; nt < 8; ++nt) {
            h1[nt][0] = h1[nt][1] = h1[nt][2] = h1[nt][3] = 0.f;
            const __nv_bfloat16 *wr = w1s + (nt * 8 + g) * 16;
            uint32_t b[2] = {*reinterpret_cast<const uint32_t *>(wr + q * 2),
                             *reinterpret_cast<const uint32_t *>(wr + 8 + q * 2)};
            mma_bf16(h1[nt], a1, b);
            const int c = nt * 8 + q * 2;
            h1[nt][0] = fmaxf(h1[nt][0] + b1s[c], 0.f);
            h1[nt][1] = fmaxf(h1[nt][1] + b1s[c + 1], 0.f);
            h1[nt][2] = fmaxf(h1[nt][2] + b1s[c], 0.f);
            h1[nt][3] = fmaxf(h1[nt][3] + b1s[c + 1], 0.f);
        }
        float h2[8][4];
#pragma unroll
        for (int nt = 0; nt < 8; ++nt) h2[nt][0] = h2[nt][1] = h2[nt][2] = h2[nt][3] = 0.f;
#pragma unroll
        for (int kb = 0; kb < 4; ++kb) {
            uint32_t a[4] = {pack_bf16(h1[2 * kb][0], h1[2 * kb][1]), pack_bf16(h1[2 * kb][2], h1[2 * kb][3]),
                             pack_bf16(h1[2 * kb + 1][0], h1[2 * kb + 1][1]),
                             pack_bf16(h1[2 * kb + 1][2], h1[2 * kb + 1][3])};
#pragma unroll
            for (int nt = 0; nt < 8; ++nt) {
                const __nv_bfloat16 *wr = w2s + (nt * 8 + g) * PH + kb * 16;
                uint32_t b[2] = {*reinterpret_cast<const uint32_t *>(wr + q * 2),
                                 *reinterpret_cast<const uint32_t *>(wr + 8 + q * 2)};
                mma_bf16(h2[nt], a, b);
            }
        }
        float y0 = 0.f, y1 = 0.f;
#pragma unroll
        for (int nt = 0; nt < 8; ++nt) {
            const int c = nt * 8 + q * 2;
            h2[nt][0] = fmaxf(h2[nt][0] + b2s[c], 0.f);
            h2[nt][1] = fmaxf(h2[nt][1] + b2s[c + 1], 0.f);
            h2[nt][2] = fmaxf(h2[nt][2] + b2s[c], 0.f);
            h2[nt][3] = fmaxf(h2[nt][3] + b2s[c + 1], 0.f);
            y0 += h2[nt][0] * w3s[c] + h2[nt][1] * w3s[c + 1];
            y1 += h2[nt][2] * w3s[c] + h2[nt][3] * w3s[c + 1];
        }
        y0 += __shfl_xor_sync(FULL, y0, 1);
        y0 += __shfl_xor_sync(FULL, y0, 2);
        y1 += __shfl_xor_sync(FULL, y1, 1);
        y1 += __shfl_xor_sync(FULL, y1, 2);
        y0 += b3s;
        y1 += b3s;
        if (mode == 1 || mode == 3) {
            float *X = p.act, *H1 = X + P_TRAIN * PF, *H2 = H1 + P_TRAIN * PH, *Y = H2 + P_TRAIN * PH,
                  *T = Y + P_TRAIN;
#pragma unroll
            for (int h = 0; h < 2; ++h) {
                const uint32_t s = sid[h];
                if (s >= n) continue;
                if (q == 0) {
#pragma unroll
                    for (int f = 0; f < PF; ++f) X[s * PF + f] = xr[h][f];
                    Y[s] = h ? y1 : y0;
                    if (mode == 1) T[s] = tr[h];
                }
#pragma unroll
                for (int nt = 0; nt < 8; ++nt) {
                    const int c = nt * 8 + q * 2;
                    // layer 2 consumed BF16(h1): keep that value for the gradient
                    H1[s * PH + c] = __bfloat162float(__float2bfloat16_rn(h1[nt][2 * h]));
                    H1[s * PH + c + 1] = __bfloat162float(__float2bfloat16_rn(h1[nt][2 * h + 1]));
                    H2[s * PH + c] = h2[nt][2 * h];
                    H2[s * PH + c + 1] = h2[nt][2 * h + 1];
                }
            }
        } else if (q == 0) {
            float *out = mode == 2 ? yout : p.scores;
            if (sid[0] < n) out[sid[0]] = y0;
            if (sid[1] < n) out[sid[1]] = y1;
        }
    }
}

// ---- backward (FP32) ----------------------------------------------------------------
// grad layout = packed params.  Loss = mean over samples of (y - t)^2.
// dz2[s][j] = 2 (y - t) / S * w3[j] * [h2 > 0];  dh1[s][k] = sum_j dz2[s][j] W2[j][k];
// dz1 = dh1 * [h1 > 0].  The weights used are the BF16 copies the forward used.
// One kernel: a block walks tiles of PB samples; per tile dz2 and dz1 are made
// in shared memory, and each thread adds the tile's terms of its parameters
// (tid, tid + 256, ...) to registers; the block adds its sums to the global
// gradient once at the end, and its share of the squared error to loss[1].
constexpr int PB = 16;                                  // samples per tile
constexpr int P_PER_THREAD = (P_NPARAM + 255) / 256;    // parameters per thread (256 threads)

__global__ void __launch_bounds__(256) pred_backward(PredDev p, uint32_t S) {
    const float *X = p.act, *H1 = X + P_TRAIN * PF, *H2 = H1 + P_TRAIN * PH, *Y = H2 + P_TRAIN * PH, *T = Y + P_TRAIN;
    __shared__ float w2[PH * PH];
    __shared__ float w3[PH];
    __shared__ float d2[PB][PH], d1[PB][PH], h1[PB][PH], h2[PB][PH];
    __shared__ float xs[PB][PF], dys[PB];
    __shared__ float lsum[8];
    for (int i = threadIdx.x; i < PH * PH; i += blockDim.x) w2[i] = __bfloat162float(p.w2b[i]);
    for (int i = threadIdx.x; i < PH; i += blockDim.x) w3[i] = p.param[P_W3 + i];
    float acc[P_PER_THREAD];
#pragma unroll
    for (int r = 0; r < P_PER_THREAD; ++r) acc[r] = 0.f;
    float lacc = 0.f;
    const uint32_t n_tiles = (S + PB - 1) / PB;
    for (uint32_t tile = blockIdx.x; tile < n_tiles; tile += gridDim.x) {
        const uint32_t s0 = tile * PB;
        __syncthreads();  // w2 / w3 loaded, or the previous tile consumed
        if (threadIdx.x < PB) {
            const uint32_t s = s0 + threadIdx.x;
            const float e = s < S ? Y[s] - T[s] : 0.f;
            dys[threadIdx.x] = 2.f * e / (float)S;
            lacc += e * e;
            for (int f = 0; f < PF; ++f)  // layer 1 consumed BF16(x)
                xs[threadIdx.x][f] = s < S ? __bfloat162float(__float2bfloat16_rn(X[s * PF + f])) : 0.f;
        }
        for (uint32_t i = threadIdx.x; i < PB * PH; i += blockDim.x) {
            const uint32_t r = i / PH, j = i % PH, s = s0 + r;
            h1[r][j] = s < S ? H1[s * PH + j] : 0.f;
            h2[r][j] = s < S ? H2[s * PH + j] : 0.f;
        }
        __syncthreads();
        for (uint32_t i = threadIdx.x; i < PB * PH; i += blockDim.x) {
            const uint32_t r = i / PH, j = i % PH;
            d2[r][j] = h2[r][j] > 0.f ? dys[r] * w3[j] : 0.f;
        }
        __syncthreads();
        for (uint32_t i = threadIdx.x; i < PB * PH; i += blockDim.x) {
            const uint32_t r = i / PH, k = i % PH;
            float a = 0.f;
#pragma unroll 16
            for (int j = 0; j < PH; ++j) a += d2[r][j] * w2[j * PH + k];
            d1[r][k] = h1[r][k] > 0.f ? a : 0.f;
        }
        __syncthreads();
#pragma unroll
        for (int q = 0; q < P_PER_THREAD; ++q) {
            const uint32_t i = threadIdx.x + 256u * q;
            float a = 0.f;
            if (i < (uint32_t)P_B1) {
                const uint32_t j = i / PF, f = i % PF;
                for (int r = 0; r < PB; ++r) a += d1[r][j] * xs[r][f];
            } else if (i < (uint32_t)P_W2) {
                for (int r = 0; r < PB; ++r) a += d1[r][i - P_B1];
            } else if (i < (uint32_t)P_B2) {
                const uint32_t j = (i - P_W2) / PH, k = (i - P_W2) % PH;
                for (int r = 0; r < PB; ++r) a += d2[r][j] * h1[r][k];
            } else if (i < (uint32_t)P_W3) {
                for (int r = 0; r < PB; ++r) a += d2[r][i - P_B2];
            } else if (i < (uint32_t)P_B3) {
                for (int r = 0; r < PB; ++r) a += dys[r] * h2[r][i - P_W3];
            } else if (i < (uint32_t)P_NPARAM) {
                for (int r = 0; r < PB; ++r) a += dys[r];
            }
            acc[q] += a;
        }
    }
#pragma unroll
    for (int q = 0; q < P_PER_THREAD; ++q) {
        const uint32_t i = threadIdx.x + 256u * q;
        if (i < (uint32_t)P_NPARAM && acc[q] != 0.f) atomicAdd(&p.grad[i], acc[q]);
    }
    for (int o = 16; o > 0; o >>= 1) lacc += __shfl_xor_sync(FULL, lacc, o);
    if ((threadIdx.x & 31) == 0) lsum[threadIdx.x >> 5] = lacc;
    __syncthreads();
    if (threadIdx.x == 0) {
        float t = 0.f;
        for (int w = 0; w < (int)(blockDim.x >> 5); ++w) t += lsum[w];
        atomicAdd(&p.loss[1], t);
    }
}

// Adam (Kingma & Ba, 2015) on the FP32 master parameters; each updated weight
// of W1 / W2 is also written to its BF16 copy (the zero padding of W1's K
// dimension is written once, by pred_cast).  The first thread turns the
// summed squared error into the step's loss.
__global__ void pred_adam(PredDev p, float lr, uint32_t S) {
    const float b1 = 0.9f, b2 = 0.999f, eps = 1e-8f;
    const uint32_t t = p.state[1] + 1;
    const float c1 = 1.f - powf(b1, (float)t), c2 = 1.f - powf(b2, (float)t);
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < P_NPARAM; i += gridDim.x * blockDim.x) {
        const float g = p.grad[i];
        const float m = b1 * p.m[i] + (1.f - b1) * g;
        const float v = b2 * p.v[i] + (1.f - b2) * g * g;
        p.m[i] = m;
        p.v[i] = v;
        const float w = p.param[i] - lr * (m / c1) / (sqrtf(v / c2) + eps);
        p.param[i] = w;
        p.grad[i] = 0.f;
        if (i < (uint32_t)P_B1) p.w1b[(i / PF) * 16 + i % PF] = __float2bfloat16_rn(w);
        else if (i >= (uint32_t)P_W2 && i < (uint32_t)P_B2) p.w2b[i - P_W2] = __float2bfloat16_rn(w);
    }
    if (blockIdx.x == 0 && threadIdx.x == 0) {
        p.loss[0] = p.loss[1] / (float)S;
        p.loss[1] = 0.f;
    }
}

// BF16 copies of W1 (K padded to 16) and W2 for the forward pass.
__global__ void pred_cast(PredDev p) {
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < PH * 16 + PH * PH; i += gridDim.x * blockDim.x) {
        if (i < PH * 16) {
            const uint32_t j = i / 16, k = i % 16;
            p.w1b[i] = __float2bfloat16_rn(k < PF ? p.param[P_W1 + j * PF + k] : 0.f);
        } else {
            p.w2b[i - PH * 16] = __float2bfloat16_rn(p.param[P_W2 + (i - PH * 16)]);
        }
    }
}

__global__ void pred_step_done(PredDev p, int trained) {
    if (threadIdx.x == 0 && blockIdx.x == 0) {
        if (trained) p.state[1] += 1;
        p.state[2] += 1;
    }
}

// The batch's counts enter the ring and the counters restart for the next
// batch; the last block to finish advances the ring position.
__global__ void pred_roll(PredDev p, uint32_t *__restrict__ counts) {
    const uint32_t pos = p.state[0];
    for (uint32_t b = blockIdx.x * blockDim.x + threadIdx.x; b < STAGE_BUCKETS; b += gridDim.x * blockDim.x) {
        p.ring[pos * STAGE_BUCKETS + b] = counts[b];
        counts[b] = 0u;
    }
    __syncthreads();
    if (threadIdx.x == 0) {
        __threadfence();
        if (atomicAdd(&p.state[3], 1u) == gridDim.x - 1u) {
            p.state[3] = 0u;
            p.state[0] = (pos + 1) % P_RING;
        }
    }
}

// Top-k scores -> staged set, in one block of 1024 threads.  Each score becomes
// a 16-bit order-preserving key (sign, exponent and 7 mantissa bits) kept in
// shared memory, so the passes below read no global memory: two 256-bin
// histogram passes find the k-th largest key (one shared atomic per distinct
// bin of a warp); buckets above it are taken, then ties in bucket order until
// k.  Thread t owns buckets 64t .. 64t+63 (its bitmap words 2t, 2t+1); their
// keys are row t of the shared array, rows padded by 4 bytes so that the
// warp's row walks hit 32 different banks.  Outputs: the bitmap and per-word
// ranks and the bucket -> group map.  The first thread also ends the
// predictor step (training step count when `trained`, batches seen).
constexpr uint32_t SELECT_ROW = 66u;  // 64 keys + 2 of padding
constexpr uint32_t SELECT_SMEM = STAGE_BUCKETS / 64u * SELECT_ROW * 2u;
__device__ __forceinline__ uint32_t select_idx(uint32_t b) { return (b >> 6) * SELECT_ROW + (b & 63u); }

__global__ void __launch_bounds__(1024) pred_select(PredDev p, uint32_t k, uint32_t *__restrict__ bits,
                                                    uint32_t *__restrict__ rank, uint16_t *__restrict__ map,
                                                    int trained) {
    extern __shared__ __align__(16) uint16_t keys[];  // STAGE_BUCKETS / 64 rows of SELECT_ROW
    __shared__ uint32_t hist[256];
    __shared__ uint32_t sel_bin, sel_rem;
    __shared__ uint32_t wsum[32];
    const uint32_t tid = threadIdx.x;
    auto okey16 = [](float f) {
        const uint32_t u = __float_as_uint(f);
        return (uint16_t)(((u & 0x80000000u) ? ~u : (u | 0x80000000u)) >> 16);
    };
    // keys of all buckets, loaded 16 bytes a thread, consecutive threads on
    // consecutive buckets
    const float4 *src = reinterpret_cast<const float4 *>(p.scores);
#pragma unroll 4
    for (uint32_t v = tid; v < STAGE_BUCKETS / 4u; v += blockDim.x) {
        const float4 f = src[v];
        uint16_t *k4 = keys + select_idx(4u * v);  // four buckets of one row
        k4[0] = okey16(f.x);
        k4[1] = okey16(f.y);
        k4[2] = okey16(f.z);
        k4[3] = okey16(f.w);
    }
    // two passes: the high byte of the k-th largest key, then its low byte
    uint32_t hi = 0, remaining = k;
    for (int pass = 0; pass < 2; ++pass) {
        if (tid < 256) hist[tid] = 0;
        __syncthreads();
        for (uint32_t b = tid; b < STAGE_BUCKETS; b += blockDim.x) {  // interleaved
            const uint32_t u = keys[select_idx(b)];
            const bool in = pass == 0 || (u >> 8) == hi;
            const uint32_t bin = !in ? 256u : pass == 0 ? (u >> 8) : (u & 255u);
            const unsigned peers = __match_any_sync(FULL, bin);
            if (in && (tid & 31u) == (uint32_t)__ffs(peers) - 1u) atomicAdd(&hist[bin], (uint32_t)__popc(peers));
        }
        __syncthreads();
        if (tid < 32) {  // the bin holding the remaining-th largest key: warp-wide suffix sums
            const uint32_t lo = (31u - tid) * 8u;  // lane 0 holds the highest bins
            uint32_t c[8], tot = 0;
#pragma unroll
            for (int i = 0; i < 8; ++i) tot += (c[i] = hist[lo + i]);
            uint32_t incl = tot;  // keys in this lane's bins and all higher ones
            for (int o = 1; o < 32; o <<= 1) {
                const uint32_t v = __shfl_up_sync(FULL, incl, o);
                if (tid >= (uint32_t)o) incl += v;
            }
            const uint32_t above = incl - tot;  // keys in higher lanes' bins
            if (above < remaining && incl >= remaining) {
                uint32_t acc = above, bin = lo;
                for (int i = 7; i >= 0; --i) {
                    if (acc + c[i] >= remaining) {
                        bin = lo + (uint32_t)i;
                        break;
                    }
                    acc += c[i];
                }
                sel_bin = bin;
                sel_rem = remaining - acc;
            }
        }
        __syncthreads();
        hi = pass == 0 ? sel_bin : (hi << 8) | sel_bin;
        remaining = sel_rem;
    }
    // hi: the k-th largest key; `remaining` of the buckets with that key are
    // still needed, taken in bucket order (exclusive scan of each thread's
    // count of such buckets among its 64)
    uint32_t tie_before = 0;
    {
        uint32_t mine = 0;
        for (uint32_t i = 0; i < 64; ++i) mine += keys[tid * SELECT_ROW + i] == hi;
        uint32_t incl = mine;
        for (int o = 1; o < 32; o <<= 1) {
            const uint32_t v = __shfl_up_sync(FULL, incl, o);
            if ((tid & 31) >= (uint32_t)o) incl += v;
        }
        if ((tid & 31) == 31) wsum[tid >> 5] = incl;
        __syncthreads();
        if (tid < 32) {
            uint32_t w = wsum[tid], wi = w;
            for (int o = 1; o < 32; o <<= 1) {
                const uint32_t v = __shfl_up_sync(FULL, wi, o);
                if (tid >= (uint32_t)o) wi += v;
            }
            wsum[tid] = wi - w;
        }
        __syncthreads();
        tie_before = wsum[tid >> 5] + incl - mine;
    }
    // bitmap words: thread owns buckets tid*64 .. tid*64+63 = words 2 tid, 2 tid + 1
    uint32_t word[2] = {0u, 0u};
    for (uint32_t i = 0; i < 64; ++i) {
        const uint32_t u = keys[tid * SELECT_ROW + i];
        bool take = u > hi;
        if (u == hi) {
            take = tie_before < remaining;
            ++tie_before;
        }
        if (take) word[i >> 5] |= 1u << (i & 31u);
    }
    bits[2 * tid] = word[0];
    bits[2 * tid + 1] = word[1];
    // rank: exclusive scan of popcounts over the 2048 words
    const uint32_t c0 = __popc(word[0]), mine = c0 + __popc(word[1]);
    uint32_t incl = mine;
    for (int o = 1; o < 32; o <<= 1) {
        const uint32_t v = __shfl_up_sync(FULL, incl, o);
        if ((tid & 31) >= (uint32_t)o) incl += v;
    }
    __syncthreads();
    if ((tid & 31) == 31) wsum[tid >> 5] = incl;
    __syncthreads();
    if (tid < 32) {
        uint32_t w = wsum[tid], wi = w;
        for (int o = 1; o < 32; o <<= 1) {
            const uint32_t v = __shfl_up_sync(FULL, wi, o);
            if (tid >= (uint32_t)o) wi += v;
        }
        wsum[tid] = wi - w;
    }
    __syncthreads();
    const uint32_t r0 = wsum[tid >> 5] + incl - mine;
    rank[2 * tid] = r0;
    rank[2 * tid + 1] = r0 + c0;
    // the map, row by row into the keys' place, then out in bucket order
    uint32_t r = r0;
    for (uint32_t i = 0; i < 64; ++i) {
        const bool on = (word[i >> 5] >> (i & 31u)) & 1u;
        keys[tid * SELECT_ROW + i] = on ? (uint16_t)r++ : (uint16_t)STAGE_NONE;
    }
    __syncthreads();
    for (uint32_t b = tid; b < STAGE_BUCKETS; b += blockDim.x) map[b] = keys[select_idx(b)];
    if (tid == 0) {
        if (trained) p.state[1] += 1;
        p.state[2] += 1;
    }
}

}  // namespace ltpg

using namespace ltpg;

struct ltpg_predictor_state {
    PredDev d{};
    float *io = nullptr;  // test io buffer
    float lr = 3e-3f;
    uint32_t train_every = 1;
    uint64_t steps_host = 0;
};

namespace {
int pfail(ltpg_ctx *c, const char *msg) {
    c->err = msg;
    return LTPG_ERR_CUDA;
}
#define PCK(call)                                                 \
    do {                                                          \
        if ((call) != cudaSuccess) return pfail(c, #call " failed"); \
    } while (0)

// Xavier-uniform initial weights from a splitmix64 stream, biases 0.
void init_params(std::vector<float> &w, uint64_t seed) {
    w.assign(P_NPARAM, 0.f);
    uint64_t s = seed;
    auto uni = [&]() {
        s += 0x9E3779B97F4A7C15ull;
        uint64_t z = s;
        z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
        z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
        z ^= z >> 31;
        return (float)((double)(z >> 11) * 0x1.0p-53 * 2.0 - 1.0);
    };
    const float a1 = sqrtf(6.f / (PF + PH)), a2 = sqrtf(6.f / (PH + PH)), a3 = sqrtf(6.f / (PH + 1));
    for (int i = 0; i < PH * PF; ++i) w[P_W1 + i] = a1 * uni();
    for (int i = 0; i < PH * PH; ++i) w[P_W2 + i] = a2 * uni();
    for (int i = 0; i < PH; ++i) w[P_W3 + i] = a3 * uni();
    for (int i = 0; i < PH; ++i) w[P_B1 + i] = 0.01f;
    for (int i = 0; i < PH; ++i) w[P_B2 + i] = 0.01f;
}
}  // namespace

extern "C" {

int ltpg_predictor_enable(ltpg_ctx *c, const ltpg_predictor_cfg *cfg) {
    if (!c || !cfg) return LTPG_ERR_INVALID;
    if (!cfg->enable) {
        c->pred_on = 0;
        c->stage_on = 0;
        drop_graphs_ctx(c);
        return LTPG_OK;
    }
    if (!c->stage_map) {
        const uint32_t none = 0;
        int r = ltpg_stage_set(c, &none, 1);  // allocates the stage arrays
        if (r) return r;
    }
    if (!c->pred) {
        ltpg_predictor_state *P = new ltpg_predictor_state();
        c->pred = P;
        PredDev &d = P->d;
        PCK(cudaMalloc(&d.param, P_NPARAM * 4));
        PCK(cudaMalloc(&d.m, P_NPARAM * 4));
        PCK(cudaMalloc(&d.v, P_NPARAM * 4));
        PCK(cudaMalloc(&d.grad, P_NPARAM * 4));
        PCK(cudaMalloc(&d.w1b, PH * 16 * 2));
        PCK(cudaMalloc(&d.w2b, PH * PH * 2));
        PCK(cudaMalloc(&d.ring, (size_t)P_RING * STAGE_BUCKETS * 4));
        PCK(cudaMalloc(&d.scores, STAGE_BUCKETS * 4));
        PCK(cudaMalloc(&d.act, (size_t)P_TRAIN * (PF + 2 * PH + 2) * 4));
        PCK(cudaMalloc(&d.state, 16));
        PCK(cudaMalloc(&d.loss, 8));
        PCK(cudaFuncSetAttribute(pred_select, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)SELECT_SMEM));
        PCK(cudaMalloc(&P->io, (size_t)P_TRAIN * 8 * 4));
    }
    ltpg_predictor_state *P = c->pred;
    std::vector<float> w;
    init_params(w, cfg->seed);
    PCK(cudaMemcpy(P->d.param, w.data(), P_NPARAM * 4, cudaMemcpyHostToDevice));
    PCK(cudaMemset(P->d.m, 0, P_NPARAM * 4));
    PCK(cudaMemset(P->d.v, 0, P_NPARAM * 4));
    PCK(cudaMemset(P->d.grad, 0, P_NPARAM * 4));
    PCK(cudaMemset(P->d.ring, 0, (size_t)P_RING * STAGE_BUCKETS * 4));
    PCK(cudaMemset(P->d.scores, 0, STAGE_BUCKETS * 4));
    PCK(cudaMemset(P->d.state, 0, 16));
    PCK(cudaMemset(P->d.loss, 0, 8));
    pred_cast<<<32, 256, 0, c->stream>>>(P->d);
    PCK(cudaGetLastError());
    P->lr = cfg->lr > 0.f ? cfg->lr : 3e-3f;
    P->train_every = cfg->train_every ? cfg->train_every : 1;
    P->steps_host = 0;
    c->pred_on = 1;
    c->pred_train = cfg->train != 0;
    c->stage_on = cfg->stage != 0;
    drop_graphs_ctx(c);
    return ltpg_sync(c);
}

int ltpg_predictor_stats(ltpg_ctx *c, float *loss, uint64_t *steps) {
    if (!c || !loss || !steps || !c->pred) return LTPG_ERR_STATE;
    uint32_t st[4];
    PCK(cudaMemcpyAsync(loss, c->pred->d.loss, 4, cudaMemcpyDeviceToHost, c->stream));
    PCK(cudaMemcpyAsync(st, c->pred->d.state, 16, cudaMemcpyDeviceToHost, c->stream));
    int r = ltpg_sync(c);
    if (r) return r;
    *steps = st[1];
    return LTPG_OK;
}

int ltpg_predictor_get_params(ltpg_ctx *c, float *host, size_t n) {
    if (!c || !host || !c->pred || n < (size_t)P_NPARAM) return LTPG_ERR_INVALID;
    PCK(cudaMemcpyAsync(host, c->pred->d.param, P_NPARAM * 4, cudaMemcpyDeviceToHost, c->stream));
    return ltpg_sync(c);
}

int ltpg_predictor_set_params(ltpg_ctx *c, const float *host, size_t n) {
    if (!c || !host || !c->pred || n < (size_t)P_NPARAM) return LTPG_ERR_INVALID;
    PCK(cudaMemcpyAsync(c->pred->d.param, host, P_NPARAM * 4, cudaMemcpyHostToDevice, c->stream));
    pred_cast<<<32, 256, 0, c->stream>>>(c->pred->d);
    PCK(cudaGetLastError());
    return ltpg_sync(c);
}

int ltpg_predictor_forward(ltpg_ctx *c, const float *host_x, uint32_t n, float *host_y) {
    if (!c || !host_x || !host_y || !c->pred || n == 0 || n > P_TRAIN) return LTPG_ERR_INVALID;
    ltpg_predictor_state *P = c->pred;
    PCK(cudaMemcpyAsync(P->io, host_x, (size_t)n * PF * 4, cudaMemcpyHostToDevice, c->stream));
    pred_forward<<<64, 256, 0, c->stream>>>(P->d, n, 2, P->io, P->io + P_TRAIN * PF);
    PCK(cudaGetLastError());
    PCK(cudaMemcpyAsync(host_y, P->io + P_TRAIN * PF, (size_t)n * 4, cudaMemcpyDeviceToHost, c->stream));
    return ltpg_sync(c);
}

int ltpg_predictor_gradients(ltpg_ctx *c, const float *host_x, const float *host_t, uint32_t n, float *host_grad) {
    if (!c || !host_x || !host_t || !host_grad || !c->pred || n == 0 || n > P_TRAIN) return LTPG_ERR_INVALID;
    ltpg_predictor_state *P = c->pred;
    // the training forward pass reads its samples from the ring; for a test we
    // run the given samples through the inference kernel and store the
    // activations with a host-side replay of mode 1's layout
    PCK(cudaMemcpyAsync(P->io, host_x, (size_t)n * PF * 4, cudaMemcpyHostToDevice, c->stream));
    pred_forward<<<64, 256, 0, c->stream>>>(P->d, n, 3, P->io, nullptr);
    PCK(cudaGetLastError());
    float *T = P->d.act + P_TRAIN * PF + 2 * P_TRAIN * PH + P_TRAIN;
    PCK(cudaMemcpyAsync(T, host_t, (size_t)n * 4, cudaMemcpyHostToDevice, c->stream));
    PCK(cudaMemsetAsync(P->d.grad, 0, P_NPARAM * 4, c->stream));
    pred_backward<<<64, 256, 0, c->stream>>>(P->d, n);
    PCK(cudaGetLastError());
    PCK(cudaMemcpyAsync(host_grad, P->d.grad, P_NPARAM * 4, cudaMemcpyDeviceToHost, c->stream));
    PCK(cudaMemsetAsync(P->d.grad, 0, P_NPARAM * 4, c->stream));
    PCK(cudaMemsetAsync(P->d.loss + 1, 0, 4, c->stream));
    return ltpg_sync(c);
}

}  // extern "C"

namespace ltpg {
// Enqueues one predictor step after a batch (also inside graph capture).
cudaError_t predictor_after_batch(ltpg_ctx *c) {
    ltpg_predictor_state *P = c->pred;
    if (!P || !c->pred_on) return cudaSuccess;
    // roll (and advance the ring), train, infer, select (and end the step)
    pred_roll<<<64, 256, 0, c->stream>>>(P->d, c->bucket_counts);
    count_launch(c);
    int trained = 0;
    if (c->pred_train) {
        pred_forward<<<64, 256, 0, c->stream>>>(P->d, P_TRAIN, 1, nullptr, nullptr);
        pred_backward<<<64, 256, 0, c->stream>>>(P->d, P_TRAIN);
        pred_adam<<<18, 256, 0, c->stream>>>(P->d, P->lr, P_TRAIN);
        count_launch(c, 3);
        trained = 1;
    }
    pred_forward<<<c->sm_count, 256, 0, c->stream>>>(P->d, STAGE_BUCKETS, 0, nullptr, nullptr);
    count_launch(c);
    if (c->stage_on) {
        const uint32_t ways = c->launch_y.ways ? c->launch_y.ways : 4u;
        pred_select<<<1, 1024, SELECT_SMEM, c->stream>>>(P->d, STAGE_MAX_ENTRIES / ways, c->stage_bits,
                                                         c->stage_rank, c->stage_map, trained);
    } else {
        pred_step_done<<<1, 32, 0, c->stream>>>(P->d, trained);
    }
    count_launch(c);
    return cudaGetLastError();
}
}  // namespace ltpg

namespace ltpg {
void predictor_free(ltpg_ctx *c) {
    ltpg_predictor_state *P = c->pred;
    if (!P) return;
    for (void *ptr : {(void *)P->d.param, (void *)P->d.m, (void *)P->d.v, (void *)P->d.grad, (void *)P->d.w1b,
                      (void *)P->d.w2b, (void *)P->d.ring, (void *)P->d.scores, (void *)P->d.act,
                      (void *)P->d.state, (void *)P->d.loss, (void *)P->io})
        if (ptr) cudaFree(ptr);
    delete P;
    c->pred = nullptr;
}
}  // namespace ltpg
