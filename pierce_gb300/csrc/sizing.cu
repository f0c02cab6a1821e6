// Learned output sizing: join summary features and a 32-64-64-1 FP32 MLP.
//
// The reference sizes its hash table and result buffer from a grid
// selectivity estimate (pierce/query/src/cuda/estimated_overlap.cu:8-77,
// host side pierce_overlap_main.cpp:376-501).  Here a small network predicts
// log(1 + unique pairs) of a join from 32 summary features of its two
// datasets; the join sizes its table from the prediction and falls back to
// the two-pass method when the prediction was too small.  The network never
// decides a predicate, so the pair set does not depend on it.
//
// Features (per side s = A, B at offset 15 s, then two cross features):
//   0      log(1 + number of objects)
//   1..3   log(1 + mean object box extent) in x, y, z
//   4..6   log(1 + variance of the box extent) in x, y, z
//   7..14  fraction of objects per triangle-count bin,
//          bin = clamp(floor(log2(tris) / 2) - 2, 0, 7)
//   30     log(1 + bbox-overlap count estimated from a 1% sample of A's
//          objects tested against every object box of B)
//   31     log(1 + nA nB prod_k(meanA_k + meanB_k) / V), the expected number
//          of overlapping boxes for uniform placement in the union box V
//
// Network: z = (x - x_mean) * x_scale; h1 = relu(W1 z + b1);
// h2 = relu(W2 h1 + b2); o = W3 h2 + b3; prediction = o * y_std + y_mean.
// Training minimises the mean squared error of o against the standardised
// targets with Adam (Kingma & Ba 2015) in one persistent thread block that
// keeps the weights and the activations of a 64-sample batch in shared
// memory; each epoch visits the samples in a fresh cyclic order.
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstring>
#include <vector>

#include "common.cuh"

namespace {

constexpr int NI = PIERCE_MLP_INPUTS;
constexpr int NH = PIERCE_MLP_HIDDEN;
constexpr int OW1 = 0;
constexpr int OB1 = OW1 + NH * NI;
constexpr int OW2 = OB1 + NH;
constexpr int OB2 = OW2 + NH * NH;
constexpr int OW3 = OB2 + NH;
constexpr int OB3 = OW3 + NH;
constexpr int NP = OB3 + 1;
static_assert(NP == PIERCE_MLP_PARAMS, "parameter layout");
// model array on the device: weights, then x_mean[NI], x_scale[NI], y_mean, y_std
constexpr int MX_MEAN = NP;
constexpr int MX_SCALE = NP + NI;
constexpr int MY_MEAN = NP + 2 * NI;
constexpr int MY_STD = MY_MEAN + 1;
constexpr int MODEL_FLOATS = MY_STD + 1;
static_assert(sizeof(pierce_mlp_params) == sizeof(float) * MODEL_FLOATS, "pierce_mlp_params layout");

constexpr int TB = 64;       // samples per training batch
constexpr int TT = 256;      // threads of the training block
constexpr int ZS = NI + 1;   // padded row strides (conflict-free column reads)
constexpr int HS = NH + 1;
constexpr int W_FLOATS = (NP + 3) & ~3;
constexpr size_t kTrainSmem =
    sizeof(float) * (W_FLOATS + TB * ZS + 4 * TB * HS + 3 * TB + 2 * NI + 2 + 2 * (TT / 32));

struct TrainArgs {
    const float* X;        // n x NI raw features
    const float* y;        // n raw targets (log1p pairs)
    int32_t n;
    int32_t epochs;
    float lr, beta1, beta2, eps;
    uint64_t seed;
    int64_t step0;         // Adam steps taken before this launch
    float* loss_out;       // per-epoch mean loss (training) or [0] = loss (gradient)
    float* grad_out;       // gradient mode: NP floats (mean over the n samples)
};

__device__ __forceinline__ uint64_t mix64(uint64_t z) {
    z += 0x9E3779B97F4A7C15ULL;
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ULL;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBULL;
    return z ^ (z >> 31);
}

// Training (UPDATE) or full-batch gradient (!UPDATE) over the samples.
template <bool UPDATE>
__global__ void __launch_bounds__(TT, 1) k_mlp_train(float* __restrict__ model, float* __restrict__ adam, TrainArgs a) {
    extern __shared__ float sm[];
    float* W = sm;
    float* Z = W + W_FLOATS;
    float* H1 = Z + TB * ZS;
    float* H2 = H1 + TB * HS;
    float* D2 = H2 + TB * HS;
    float* D1 = D2 + TB * HS;
    float* O = D1 + TB * HS;
    float* DO = O + TB;
    float* T = DO + TB;
    float* xm = T + TB;
    float* xs = xm + NI;
    float* yn = xs + NI;  // y_mean, y_std
    float* red = yn + 2;  // per-warp loss partials (2 x warps)
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    constexpr int NW = TT / 32;

    for (int p = tid; p < NP; p += TT) W[p] = model[p];
    for (int k = tid; k < NI; k += TT) {
        xm[k] = model[MX_MEAN + k];
        xs[k] = model[MX_SCALE + k];
    }
    if (tid == 0) {
        yn[0] = model[MY_MEAN];
        yn[1] = model[MY_STD];
    }
    __syncthreads();
    const float inv_ystd = yn[1] != 0.0f ? 1.0f / yn[1] : 1.0f;

    const int n = a.n;
    const int epochs = UPDATE ? a.epochs : 1;
    const int batches = (n + TB - 1) / TB;
    int64_t step = a.step0;
    static const uint32_t kStrides[8] = {1000003u, 1299709u, 1500007u, 1700021u,
                                         1900009u, 2000003u, 2500009u, 2999999u};
    for (int ep = 0; ep < epochs; ++ep) {
        // cyclic visiting order of this epoch: (offset + i * stride) mod n,
        // stride a prime larger than n so every sample is visited once
        const uint64_t h = mix64(a.seed ^ (0x5851F42D4C957F2DULL * (uint64_t)(ep + 1)));
        const uint64_t stride = UPDATE ? kStrides[h & 7] : 1;
        const uint64_t offset = UPDATE ? (h >> 8) % (uint64_t)n : 0;
        float epoch_loss = 0.0f;  // thread 0 only
        for (int bt = 0; bt < batches; ++bt) {
            const int b0 = bt * TB;
            const int nb = min(TB, n - b0);
            // 1. standardised inputs and targets
            for (int e = tid; e < TB * NI; e += TT) {
                const int b = e / NI, k = e % NI;
                float z = 0.0f;
                if (b < nb) {
                    const uint64_t s = (offset + (uint64_t)(b0 + b) * stride) % (uint64_t)n;
                    z = (a.X[s * NI + k] - xm[k]) * xs[k];
                }
                Z[b * ZS + k] = z;
            }
            if (tid < TB) {
                float t = 0.0f;
                if (tid < nb) {
                    const uint64_t s = (offset + (uint64_t)(b0 + tid) * stride) % (uint64_t)n;
                    t = (a.y[s] - yn[0]) * inv_ystd;
                }
                T[tid] = t;
            }
            __syncthreads();
            // 2. h1 = relu(W1 z + b1): lanes over samples, warps over units
            for (int j = warp; j < NH; j += NW) {
                const float* w = W + OW1 + j * NI;
                float acc0 = W[OB1 + j], acc1 = acc0;
#pragma unroll 8
                for (int k = 0; k < NI; ++k) {
                    acc0 = fmaf(w[k], Z[lane * ZS + k], acc0);
                    acc1 = fmaf(w[k], Z[(lane + 32) * ZS + k], acc1);
                }
                H1[lane * HS + j] = fmaxf(acc0, 0.0f);
                H1[(lane + 32) * HS + j] = fmaxf(acc1, 0.0f);
            }
            __syncthreads();
            // 3. h2 = relu(W2 h1 + b2)
            for (int j = warp; j < NH; j += NW) {
                const float* w = W + OW2 + j * NH;
                float acc0 = W[OB2 + j], acc1 = acc0;
#pragma unroll 8
                for (int k = 0; k < NH; ++k) {
                    acc0 = fmaf(w[k], H1[lane * HS + k], acc0);
                    acc1 = fmaf(w[k], H1[(lane + 32) * HS + k], acc1);
                }
                H2[lane * HS + j] = fmaxf(acc0, 0.0f);
                H2[(lane + 32) * HS + j] = fmaxf(acc1, 0.0f);
            }
            __syncthreads();
            // 4. output, loss and its derivative (mean over the batch when
            // training, over all n samples for the full-batch gradient)
            if (tid < TB) {
                float acc = W[OB3];
#pragma unroll 8
                for (int k = 0; k < NH; ++k) acc = fmaf(W[OW3 + k], H2[tid * HS + k], acc);
                O[tid] = acc;
                const float r = tid < nb ? acc - T[tid] : 0.0f;
                DO[tid] = 2.0f * r / (float)(UPDATE ? nb : n);
                float l = r * r;
                for (int off = 16; off > 0; off >>= 1) l += __shfl_xor_sync(0xFFFFFFFFu, l, off);
                if (lane == 0) red[warp] = l;
            }
            __syncthreads();
            if (tid == 0) epoch_loss += red[0] + red[1];
            // 5. d h2 = dO W3 relu'(h2)
            for (int e = tid; e < TB * NH; e += TT) {
                const int b = e / NH, j = e % NH;
                D2[b * HS + j] = H2[b * HS + j] > 0.0f ? DO[b] * W[OW3 + j] : 0.0f;
            }
            __syncthreads();
            // 6. d h1 = (W2^T d h2) relu'(h1): lanes over samples, warps over units
            for (int k = warp; k < NH; k += NW) {
                float acc0 = 0.0f, acc1 = 0.0f;
#pragma unroll 8
                for (int j = 0; j < NH; ++j) {
                    const float w = W[OW2 + j * NH + k];
                    acc0 = fmaf(w, D2[lane * HS + j], acc0);
                    acc1 = fmaf(w, D2[(lane + 32) * HS + j], acc1);
                }
                D1[lane * HS + k] = H1[lane * HS + k] > 0.0f ? acc0 : 0.0f;
                D1[(lane + 32) * HS + k] = H1[(lane + 32) * HS + k] > 0.0f ? acc1 : 0.0f;
            }
            __syncthreads();
            // 7. parameter gradients (sums over the batch), then Adam or accumulation
            ++step;
            const float bc1 = 1.0f - powf(a.beta1, (float)step);
            const float bc2 = 1.0f - powf(a.beta2, (float)step);
            for (int p = tid; p < NP; p += TT) {
                float g = 0.0f;
                if (p < OB1) {  // W1[j][k]
                    const int j = p / NI, k = p % NI;
                    for (int b = 0; b < TB; ++b) g = fmaf(D1[b * HS + j], Z[b * ZS + k], g);
                } else if (p < OW2) {  // b1
                    const int j = p - OB1;
                    for (int b = 0; b < TB; ++b) g += D1[b * HS + j];
                } else if (p < OB2) {  // W2[j][k]
                    const int q = p - OW2, j = q / NH, k = q % NH;
                    for (int b = 0; b < TB; ++b) g = fmaf(D2[b * HS + j], H1[b * HS + k], g);
                } else if (p < OW3) {  // b2
                    const int j = p - OB2;
                    for (int b = 0; b < TB; ++b) g += D2[b * HS + j];
                } else if (p < OB3) {  // W3
                    const int k = p - OW3;
                    for (int b = 0; b < TB; ++b) g = fmaf(DO[b], H2[b * HS + k], g);
                } else {  // b3
                    for (int b = 0; b < TB; ++b) g += DO[b];
                }
                if (UPDATE) {
                    float m = adam[p], v = adam[NP + p];
                    m = a.beta1 * m + (1.0f - a.beta1) * g;
                    v = a.beta2 * v + (1.0f - a.beta2) * g * g;
                    adam[p] = m;
                    adam[NP + p] = v;
                    W[p] -= a.lr * (m / bc1) / (sqrtf(v / bc2) + a.eps);
                } else {
                    a.grad_out[p] += g;
                }
            }
            __syncthreads();
        }
        if (tid == 0 && a.loss_out) a.loss_out[ep] = epoch_loss / (float)n;
    }
    if (UPDATE)
        for (int p = tid; p < NP; p += TT) model[p] = W[p];
}

// Inference: one 64-thread block per sample; out = log1p(pairs) prediction.
__global__ void __launch_bounds__(NH) k_mlp_predict(const float* __restrict__ model, const float* __restrict__ X,
                                                    int32_t n, float* __restrict__ out) {
    __shared__ float z[NI], h1[NH], part[NH / 32];
    __shared__ float h2[NH];
    const int j = threadIdx.x;
    for (int s = blockIdx.x; s < n; s += gridDim.x) {
        if (j < NI) z[j] = (X[(size_t)s * NI + j] - model[MX_MEAN + j]) * model[MX_SCALE + j];
        __syncthreads();
        float acc = model[OB1 + j];
        for (int k = 0; k < NI; ++k) acc = fmaf(model[OW1 + j * NI + k], z[k], acc);
        h1[j] = fmaxf(acc, 0.0f);
        __syncthreads();
        acc = model[OB2 + j];
        for (int k = 0; k < NH; ++k) acc = fmaf(model[OW2 + j * NH + k], h1[k], acc);
        h2[j] = fmaxf(acc, 0.0f);
        float o = model[OW3 + j] * h2[j];
        for (int off = 16; off > 0; off >>= 1) o += __shfl_xor_sync(0xFFFFFFFFu, o, off);
        if ((j & 31) == 0) part[j >> 5] = o;
        __syncthreads();
        if (j == 0) {
            const float t = part[0] + part[1] + model[OB3];
            out[s] = t * model[MY_STD] + model[MY_MEAN];
        }
        __syncthreads();
    }
}

// Per-feature mean and 1/std of the inputs and mean/std of the targets
// (one block of NI threads; thread NI-1.. handles y after its feature).
__global__ void k_fit_normalization(const float* __restrict__ X, const float* __restrict__ y, int32_t n,
                                    float* __restrict__ model) {
    const int k = threadIdx.x;
    if (k <= NI) {
        double s = 0.0, s2 = 0.0;
        for (int32_t i = 0; i < n; ++i) {
            const double v = k < NI ? X[(size_t)i * NI + k] : y[i];
            s += v;
            s2 += v * v;
        }
        const double mean = n ? s / n : 0.0;
        const double var = n ? fmax(s2 / n - mean * mean, 0.0) : 0.0;
        const double sd = sqrt(var);
        if (k < NI) {
            model[MX_MEAN + k] = (float)mean;
            model[MX_SCALE + k] = sd > 1e-6 ? (float)(1.0 / sd) : 1.0f;
        } else {
            model[MY_MEAN] = (float)mean;
            model[MY_STD] = sd > 1e-6 ? (float)sd : 1.0f;
        }
    }
}

// ---- features -----------------------------------------------------------------

// Per-object triangle counts (warp-aggregated when a warp's triangles share
// one object, which is the common case: objects are contiguous).
__global__ void k_obj_tri_counts(const int32_t* __restrict__ t2o, int64_t nt, int32_t nobj,
                                 unsigned int* __restrict__ counts) {
    const int64_t stride = (int64_t)gridDim.x * blockDim.x;
    for (int64_t base = blockIdx.x * (int64_t)blockDim.x; base < nt; base += stride) {
        const int64_t t = base + threadIdx.x;
        int32_t o = t < nt ? t2o[t] : -1;
        if (o >= nobj) o = -1;
        const int32_t o0 = __shfl_sync(0xFFFFFFFFu, o, 0);
        const unsigned valid = __ballot_sync(0xFFFFFFFFu, o >= 0);
        if (__all_sync(0xFFFFFFFFu, o == o0 || o < 0) && o0 >= 0) {
            if ((threadIdx.x & 31) == 0) atomicAdd(counts + o0, (unsigned)__popc(valid));
        } else if (o >= 0) {
            atomicAdd(counts + o, 1u);
        }
    }
}

// Per-object triangle counts of a dataset whose objects are stored
// contiguously: the count of each object's triangle range (no atomics; a
// long object would otherwise have thousands of warps add to one counter).
__global__ void k_obj_counts_from_ranges(const int2* __restrict__ ranges, int32_t nobj,
                                         unsigned int* __restrict__ counts) {
    for (int64_t o = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; o < nobj; o += (int64_t)gridDim.x * blockDim.x)
        counts[o] = (unsigned int)__ldg(&ranges[o].y);
}

// Side statistics: acc[0] valid objects, [1..3] sum extent, [4..6] sum
// extent^2, [7..14] histogram; bounds (ordered-int lo[3], hi[3]).
constexpr int kAcc = 16;

__device__ __forceinline__ uint32_t f2o(float f) {
    const uint32_t u = __float_as_uint(f);
    return (u & 0x80000000u) ? ~u : (u | 0x80000000u);
}
__device__ __forceinline__ float o2f(uint32_t u) {
    return __uint_as_float((u & 0x80000000u) ? (u & 0x7FFFFFFFu) : ~u);
}

__global__ void k_side_stats(const float* __restrict__ box, const unsigned int* __restrict__ counts, int32_t nobj,
                             double* __restrict__ acc, uint32_t* __restrict__ bounds) {
    double v[15];
    for (int k = 0; k < 15; ++k) v[k] = 0.0;
    float lo[3] = {3.4e38f, 3.4e38f, 3.4e38f}, hi[3] = {-3.4e38f, -3.4e38f, -3.4e38f};
    for (int64_t o = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; o < nobj; o += (int64_t)gridDim.x * blockDim.x) {
        const unsigned c = counts[o];
        if (c == 0) continue;
        const float* b = box + 6 * o;
        v[0] += 1.0;
        for (int k = 0; k < 3; ++k) {
            const double e = (double)b[3 + k] - (double)b[k];
            v[1 + k] += e;
            v[4 + k] += e * e;
            lo[k] = fminf(lo[k], b[k]);
            hi[k] = fmaxf(hi[k], b[3 + k]);
        }
        const int bin = min(max((31 - __clz(c)) / 2 - 2, 0), 7);
        v[7 + bin] += 1.0;
    }
    for (int k = 0; k < 15; ++k) {
        for (int off = 16; off > 0; off >>= 1) v[k] += __shfl_xor_sync(0xFFFFFFFFu, v[k], off);
        if ((threadIdx.x & 31) == 0 && v[k] != 0.0) atomicAdd(acc + k, v[k]);
    }
    for (int k = 0; k < 3; ++k) {
        for (int off = 16; off > 0; off >>= 1) {
            lo[k] = fminf(lo[k], __shfl_xor_sync(0xFFFFFFFFu, lo[k], off));
            hi[k] = fmaxf(hi[k], __shfl_xor_sync(0xFFFFFFFFu, hi[k], off));
        }
        if ((threadIdx.x & 31) == 0) {
            atomicMin(bounds + k, f2o(lo[k]));
            atomicMax(bounds + 3 + k, f2o(hi[k]));
        }
    }
}

// Sampled box-overlap count: every `step`-th object of A against all of B.
constexpr int kSampleTile = 256;

__global__ void __launch_bounds__(256) k_sample_overlap(const float* __restrict__ box_a,
                                                        const unsigned int* __restrict__ cnt_a, int32_t na,
                                                        int32_t step, const float* __restrict__ box_b,
                                                        const unsigned int* __restrict__ cnt_b, int32_t nb,
                                                        unsigned long long* __restrict__ out) {
    __shared__ float tile[kSampleTile * 6];
    const int32_t ns = (na + step - 1) / step;
    unsigned long long hits = 0;
    for (int64_t base = blockIdx.x * (int64_t)blockDim.x; base < nb; base += (int64_t)gridDim.x * blockDim.x) {
        const int64_t o = base + threadIdx.x;
        float b[6] = {3.4e38f, 3.4e38f, 3.4e38f, -3.4e38f, -3.4e38f, -3.4e38f};  // empty unless valid
        if (o < nb && cnt_b[o] > 0)
            for (int k = 0; k < 6; ++k) b[k] = box_b[6 * o + k];
        for (int32_t t0 = 0; t0 < ns; t0 += kSampleTile) {
            const int m = min(kSampleTile, ns - t0);
            __syncthreads();
            for (int e = threadIdx.x; e < m * 6; e += blockDim.x) {
                const int64_t ia = (int64_t)(t0 + e / 6) * step;
                tile[e] = cnt_a[ia] > 0 ? box_a[6 * ia + e % 6] : ((e % 6) < 3 ? 3.4e38f : -3.4e38f);
            }
            __syncthreads();
            for (int i = 0; i < m; ++i) {
                const float* a = tile + 6 * i;
                hits += (a[0] <= b[3] && b[0] <= a[3] && a[1] <= b[4] && b[1] <= a[4] && a[2] <= b[5] &&
                         b[2] <= a[5])
                            ? 1u
                            : 0u;
            }
        }
    }
    for (int off = 16; off > 0; off >>= 1) hits += __shfl_xor_sync(0xFFFFFFFFu, hits, off);
    if ((threadIdx.x & 31) == 0 && hits) atomicAdd(out, hits);
}

__global__ void k_features_finalize(const double* __restrict__ acc, const uint32_t* __restrict__ bounds,
                                    const unsigned long long* __restrict__ sample, int32_t na, int32_t nb,
                                    int32_t step, float* __restrict__ f) {
    if (threadIdx.x != 0 || blockIdx.x != 0) return;
    const int32_t nobj[2] = {na, nb};
    double mean[2][3];
    for (int s = 0; s < 2; ++s) {
        const double* a = acc + kAcc * s;
        const double n = a[0];
        f[15 * s] = (float)log1p((double)nobj[s]);
        for (int k = 0; k < 3; ++k) {
            const double m = n > 0 ? a[1 + k] / n : 0.0;
            const double var = n > 0 ? fmax(a[4 + k] / n - m * m, 0.0) : 0.0;
            mean[s][k] = m;
            f[15 * s + 1 + k] = (float)log1p(m);
            f[15 * s + 4 + k] = (float)log1p(var);
        }
        for (int h = 0; h < 8; ++h) f[15 * s + 7 + h] = n > 0 ? (float)(a[7 + h] / n) : 0.0f;
    }
    const int32_t ns = na > 0 ? (na + step - 1) / step : 0;
    const double scaled = ns > 0 ? (double)sample[0] * (double)na / (double)ns : 0.0;
    f[30] = (float)log1p(scaled);
    double vol = 1.0;
    for (int k = 0; k < 3; ++k) {
        const double lo = fmin((double)o2f(bounds[k]), (double)o2f(bounds[6 + k]));
        const double hi = fmax((double)o2f(bounds[3 + k]), (double)o2f(bounds[9 + k]));
        vol *= fmax(hi - lo, 1e-6);
    }
    double expect = (double)na * (double)nb / vol;
    for (int k = 0; k < 3; ++k) expect *= mean[0][k] + mean[1][k];
    if (!(expect >= 0.0) || isinf(expect)) expect = 0.0;
    f[31] = (na > 0 && nb > 0) ? (float)log1p(expect) : 0.0f;
}

__global__ void k_bounds_init(uint32_t* b) {
    const int k = threadIdx.x;
    if (k < 12) b[k] = (k % 6) < 3 ? 0xFFFFFFFFu : 0u;
}

int grid_for(pierce_ctx* ctx, int64_t n, int block) {
    int64_t b = (n + block - 1) / block;
    const int64_t cap = (int64_t)ctx->sm_count * 16;
    if (b > cap) b = cap;
    return (int)(b < 1 ? 1 : b);
}

}  // namespace

struct pierce_mlp {
    pierce_ctx* ctx = nullptr;
    int device = 0;  // ctx->device, kept for release
    float* d_model = nullptr;  // MODEL_FLOATS
    float* d_adam = nullptr;   // 2 * NP (first and second moments)
    int64_t steps = 0;
};

namespace pgpu {

constexpr int kSampleStep = 100;  // 1% of A's objects

// Features of the join (A, B) into d_out[0..31] (device memory).
int join_features(pierce_ctx* ctx, const pierce_dataset* A, const pierce_dataset* B, float* d_out) {
    cudaStream_t st = ctx->stream;
    const size_t na = (size_t)std::max(A->num_objects, 0), nb = (size_t)std::max(B->num_objects, 0);
    // scratch: acc (2 x kAcc doubles), bounds (12 u32), sample count, counts A, counts B
    const size_t head = 8 * 2 * kAcc + 64 + 16;
    void* p = nullptr;
    if (int s = scratch(ctx, kSizingScratchSlot, head + 4 * (na + nb) + 16, &p)) return s;
    char* base = static_cast<char*>(p);
    double* acc = reinterpret_cast<double*>(base);
    uint32_t* bounds = reinterpret_cast<uint32_t*>(base + 8 * 2 * kAcc);
    unsigned long long* sample = reinterpret_cast<unsigned long long*>(base + 8 * 2 * kAcc + 64);
    unsigned int* cnt_a = reinterpret_cast<unsigned int*>(base + head);
    unsigned int* cnt_b = cnt_a + na;
    cudaMemsetAsync(base, 0, head + 4 * (na + nb), st);
    k_bounds_init<<<1, 32, 0, st>>>(bounds);
    int launches = 2;
    const pierce_dataset* ds[2] = {A, B};
    unsigned int* cnt[2] = {cnt_a, cnt_b};
    for (int s = 0; s < 2; ++s) {
        if (ds[s]->nt > 0 && ds[s]->num_objects > 0) {
            if (ds[s]->contiguous && ds[s]->d_obj_range)
                k_obj_counts_from_ranges<<<grid_for(ctx, ds[s]->num_objects, 256), 256, 0, st>>>(
                    ds[s]->d_obj_range, ds[s]->num_objects, cnt[s]);
            else
                k_obj_tri_counts<<<grid_for(ctx, (int64_t)ds[s]->nt, 256), 256, 0, st>>>(
                    ds[s]->d_tri_to_object, (int64_t)ds[s]->nt, ds[s]->num_objects, cnt[s]);
            k_side_stats<<<grid_for(ctx, ds[s]->num_objects, 256), 256, 0, st>>>(
                ds[s]->d_obj_box, cnt[s], ds[s]->num_objects, acc + kAcc * s, bounds + 6 * s);
            launches += 2;
        }
    }
    if (na > 0 && nb > 0) {
        k_sample_overlap<<<grid_for(ctx, (int64_t)nb, 256), 256, 0, st>>>(A->d_obj_box, cnt_a, (int32_t)na,
                                                                         kSampleStep, B->d_obj_box, cnt_b,
                                                                         (int32_t)nb, sample);
        ++launches;
    }
    k_features_finalize<<<1, 32, 0, st>>>(acc, bounds, sample, (int32_t)na, (int32_t)nb, kSampleStep, d_out);
    ctx->launches += launches + 1;
    return check_cuda(cudaGetLastError(), "join features");
}

// Predicted log1p(pairs) of the join into *pred (synchronous), capped by the
// sampled box-overlap estimate.
int learned_log_pairs(pierce_ctx* ctx, const pierce_mlp* mlp, const pierce_dataset* A, const pierce_dataset* B,
                      double* pred) {
    void* p = nullptr;
    if (int s = scratch(ctx, kSizingScratchSlot + 1, 64 * sizeof(float), &p)) return s;
    float* f = static_cast<float*>(p);
    if (int s = join_features(ctx, A, B, f)) return s;
    k_mlp_predict<<<1, NH, 0, ctx->stream>>>(mlp->d_model, f, 1, f + NI);
    ctx->launches += 1;
    int64_t bits = 0, sample_bits = 0;
    if (int s = host_value(ctx, f + NI, 4, &bits, "learned sizing")) return s;
    if (int s = host_value(ctx, f + 30, 4, &sample_bits, "learned sizing bound")) return s;
    const int32_t b32 = (int32_t)bits, s32 = (int32_t)sample_bits;
    float v, sv;
    std::memcpy(&v, &b32, sizeof(float));
    std::memcpy(&sv, &s32, sizeof(float));
    // Outside its training distribution the network can predict far more
    // pairs than can exist: cap it by 4x the sampled box-overlap estimate
    // (every pair is a box overlap) plus a floor, and by nA nB.  A cap below
    // the true count only costs the two-pass rerun.
    const double boxes = std::expm1((double)sv);
    const double cap = std::min(4.0 * boxes + 4096.0, (double)A->num_objects * (double)B->num_objects + 1.0);
    *pred = std::min((double)v, std::log1p(cap));
    return PIERCE_OK;
}

}  // namespace pgpu

using namespace pgpu;

namespace {

int upload(pierce_ctx* ctx, const void* host, size_t bytes, void** dev, const char* what) {
    if (int s = device_alloc(dev, std::max<size_t>(bytes, 16), what)) return s;
    if (bytes) return check_cuda(cudaMemcpyAsync(*dev, host, bytes, cudaMemcpyHostToDevice, ctx->stream), what);
    return PIERCE_OK;
}

}  // namespace

extern "C" {

void pierce_default_mlp_train_opts(pierce_mlp_train_opts* o) {
    if (!o) return;
    o->epochs = 400;
    o->lr = 1e-3f;
    o->beta1 = 0.9f;
    o->beta2 = 0.999f;
    o->eps = 1e-8f;
    o->seed = 1;
    o->fit_normalization = 1;
}

int pierce_mlp_init_params(pierce_mlp_params* p, uint64_t seed) {
    if (!p) return set_error(PIERCE_ERR_INVALID_ARGUMENT, "mlp_init_params: null argument");
    std::memset(p, 0, sizeof(*p));
    // He-uniform weights, zero biases; a splitmix stream gives the uniforms.
    uint64_t x = seed;
    auto uniform = [&x]() {
        uint64_t z = (x += 0x9E3779B97F4A7C15ULL);
        z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ULL;
        z = (z ^ (z >> 27)) * 0x94D049BB133111EBULL;
        z ^= z >> 31;
        return (double)(z >> 11) * (1.0 / 9007199254740992.0);
    };
    auto fill = [&](int off, int fan_out, int fan_in) {
        const double lim = std::sqrt(6.0 / fan_in);
        for (int i = 0; i < fan_out * fan_in; ++i) p->weights[off + i] = (float)((2.0 * uniform() - 1.0) * lim);
    };
    fill(OW1, NH, NI);
    fill(OW2, NH, NH);
    fill(OW3, 1, NH);
    for (int k = 0; k < NI; ++k) p->x_scale[k] = 1.0f;
    p->y_std = 1.0f;
    return PIERCE_OK;
}

int pierce_mlp_create(pierce_ctx* ctx, const pierce_mlp_params* init, pierce_mlp** out) {
    if (!ctx || !init || !out) return set_error(PIERCE_ERR_INVALID_ARGUMENT, "mlp_create: null argument");
    *out = nullptr;
    cudaSetDevice(ctx->device);
    pierce_mlp* m = new pierce_mlp();
    m->ctx = ctx;
    m->device = ctx->device;
    int s = PIERCE_OK;
    do {
        if ((s = device_alloc((void**)&m->d_model, sizeof(float) * MODEL_FLOATS, "mlp model"))) break;
        if ((s = device_alloc((void**)&m->d_adam, sizeof(float) * 2 * NP, "mlp optimiser state"))) break;
        cudaMemcpyAsync(m->d_model, init, sizeof(float) * MODEL_FLOATS, cudaMemcpyHostToDevice, ctx->stream);
        cudaMemsetAsync(m->d_adam, 0, sizeof(float) * 2 * NP, ctx->stream);
        s = check_cuda(cudaStreamSynchronize(ctx->stream), "mlp create");
    } while (0);
    if (s) {
        pierce_mlp_destroy(m);
        return s;
    }
    *out = m;
    return PIERCE_OK;
}

void pierce_mlp_destroy(pierce_mlp* m) {
    if (!m) return;
    cudaSetDevice(m->device);
    cudaDeviceSynchronize();
    if (m->d_model) cudaFree(m->d_model);
    if (m->d_adam) cudaFree(m->d_adam);
    delete m;
}

int pierce_mlp_get(pierce_ctx* ctx, const pierce_mlp* m, pierce_mlp_params* out) {
    if (!ctx || !m || !out) return set_error(PIERCE_ERR_INVALID_ARGUMENT, "mlp_get: null argument");
    cudaMemcpyAsync(out, m->d_model, sizeof(float) * MODEL_FLOATS, cudaMemcpyDeviceToHost, ctx->stream);
    return check_cuda(cudaStreamSynchronize(ctx->stream), "mlp get");
}

static int run_train(pierce_ctx* ctx, pierce_mlp* m, const float* X, const float* y, int32_t n,
                     const pierce_mlp_train_opts* opts, float* loss_host, float* grad_host, bool update) {
    if (!ctx || !m || n <= 0 || !X || !y || (n > (1 << 20)))
        return set_error(PIERCE_ERR_INVALID_ARGUMENT, "mlp train: invalid argument (0 < n <= 2^20)");
    pierce_mlp_train_opts o;
    pierce_default_mlp_train_opts(&o);
    if (opts) o = *opts;
    if (update && (o.epochs <= 0 || !(o.lr > 0.0f)))
        return set_error(PIERCE_ERR_INVALID_ARGUMENT, "mlp train: epochs and learning rate must be positive");
    cudaSetDevice(ctx->device);
    cudaStream_t st = ctx->stream;
    void *dx = nullptr, *dy = nullptr, *dl = nullptr, *dg = nullptr;
    const int nloss = update ? o.epochs : 1;
    int s = PIERCE_OK;
    do {
        if ((s = upload(ctx, X, sizeof(float) * NI * (size_t)n, &dx, "mlp inputs"))) break;
        if ((s = upload(ctx, y, sizeof(float) * (size_t)n, &dy, "mlp targets"))) break;
        if ((s = device_alloc(&dl, sizeof(float) * nloss, "mlp losses"))) break;
        if (!update) {
            if ((s = device_alloc(&dg, sizeof(float) * NP, "mlp gradient"))) break;
            cudaMemsetAsync(dg, 0, sizeof(float) * NP, st);
        }
        if (update && o.fit_normalization) {
            k_fit_normalization<<<1, NI + 1, 0, st>>>((const float*)dx, (const float*)dy, n, m->d_model);
            ctx->launches += 1;
        }
        TrainArgs a;
        a.X = (const float*)dx;
        a.y = (const float*)dy;
        a.n = n;
        a.epochs = o.epochs;
        a.lr = o.lr;
        a.beta1 = o.beta1;
        a.beta2 = o.beta2;
        a.eps = o.eps;
        a.seed = o.seed;
        a.step0 = m->steps;
        a.loss_out = (float*)dl;
        a.grad_out = (float*)dg;
        if (update) {
            if ((s = check_cuda(cudaFuncSetAttribute(k_mlp_train<true>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                                     (int)kTrainSmem),
                                "mlp smem")))
                break;
            k_mlp_train<true><<<1, TT, kTrainSmem, st>>>(m->d_model, m->d_adam, a);
            m->steps += (int64_t)o.epochs * ((n + TB - 1) / TB);
        } else {
            if ((s = check_cuda(cudaFuncSetAttribute(k_mlp_train<false>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                                     (int)kTrainSmem),
                                "mlp smem")))
                break;
            k_mlp_train<false><<<1, TT, kTrainSmem, st>>>(m->d_model, m->d_adam, a);
        }
        ctx->launches += 1;
        if ((s = check_cuda(cudaGetLastError(), "mlp train launch"))) break;
        if (loss_host) cudaMemcpyAsync(loss_host, dl, sizeof(float) * nloss, cudaMemcpyDeviceToHost, st);
        if (grad_host) cudaMemcpyAsync(grad_host, dg, sizeof(float) * NP, cudaMemcpyDeviceToHost, st);
        s = check_cuda(cudaStreamSynchronize(st), "mlp train");
    } while (0);
    cudaStreamSynchronize(st);
    for (void* q : {dx, dy, dl, dg})
        if (q) cudaFree(q);
    return s;
}

int pierce_mlp_train(pierce_ctx* ctx, pierce_mlp* m, const float* X, const float* y, int32_t n,
                     const pierce_mlp_train_opts* opts, float* loss_per_epoch) {
    return run_train(ctx, m, X, y, n, opts, loss_per_epoch, nullptr, true);
}

int pierce_mlp_gradient(pierce_ctx* ctx, const pierce_mlp* m, const float* X, const float* y, int32_t n,
                        float* grad, float* loss) {
    if (!grad) return set_error(PIERCE_ERR_INVALID_ARGUMENT, "mlp_gradient: null gradient");
    return run_train(ctx, const_cast<pierce_mlp*>(m), X, y, n, nullptr, loss, grad, false);
}

int pierce_mlp_predict(pierce_ctx* ctx, const pierce_mlp* m, const float* X, int32_t n, float* out) {
    if (!ctx || !m || n < 0 || (n && (!X || !out)))
        return set_error(PIERCE_ERR_INVALID_ARGUMENT, "mlp_predict: invalid argument");
    if (n == 0) return PIERCE_OK;
    cudaSetDevice(ctx->device);
    void *dx = nullptr, *dout = nullptr;
    int s = PIERCE_OK;
    do {
        if ((s = upload(ctx, X, sizeof(float) * NI * (size_t)n, &dx, "mlp inputs"))) break;
        if ((s = device_alloc(&dout, sizeof(float) * (size_t)n, "mlp outputs"))) break;
        k_mlp_predict<<<std::min(n, 65535), NH, 0, ctx->stream>>>(m->d_model, (const float*)dx, n, (float*)dout);
        ctx->launches += 1;
        if ((s = check_cuda(cudaGetLastError(), "mlp predict launch"))) break;
        cudaMemcpyAsync(out, dout, sizeof(float) * (size_t)n, cudaMemcpyDeviceToHost, ctx->stream);
        s = check_cuda(cudaStreamSynchronize(ctx->stream), "mlp predict");
    } while (0);
    cudaStreamSynchronize(ctx->stream);
    for (void* q : {dx, dout})
        if (q) cudaFree(q);
    return s;
}

int pierce_join_features(pierce_ctx* ctx, const pierce_dataset* a, const pierce_dataset* b, float* out) {
    if (!ctx || !a || !b || !out) return set_error(PIERCE_ERR_INVALID_ARGUMENT, "join_features: null argument");
    cudaSetDevice(ctx->device);
    void* p = nullptr;
    if (int s = scratch(ctx, kSizingScratchSlot + 1, 64 * sizeof(float), &p)) return s;
    if (int s = join_features(ctx, a, b, static_cast<float*>(p))) return s;
    cudaMemcpyAsync(out, p, sizeof(float) * NI, cudaMemcpyDeviceToHost, ctx->stream);
    return check_cuda(cudaStreamSynchronize(ctx->stream), "join features");
}

}  // extern "C"
