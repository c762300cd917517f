// Learned per-level variant switching: profiling, the MLP (FP32, hand-written
// training and inference kernels) and the switched traversal.
#include <algorithm>
#include <cmath>
#include <cstring>
#include <vector>

#include "bw_features.h"
#include "bw_hash.h"
#include "bw_internal.cuh"

namespace bw {

// Implemented in bfs.cu (shared with the fixed-variant paths).
int bfs_prepare(bw_context *ctx, const bw_graph_view *g, int reps, bool side, int32_t *levels,
                uint32_t root, cudaStream_t s);
int bfs_plan(const bw_context *ctx, int variant, bool side, const bw_launch_config *cfg, BfsKernelFn *k,
             BfsKernelFn *k2, unsigned *block, unsigned *grid, size_t *smem);
BfsArgs bfs_args(bw_context *ctx, const bw_graph_view *g, int32_t *levels, int32_t depth,
                 const bw_launch_config *cfg);
int bfs_variant_reps(int v);
int bfs_traversed(bw_context *ctx, const bw_graph_view *g, int32_t *levels, cudaStream_t s, uint64_t *out);
__global__ void k_bfs_init_side(int32_t *levels, uint64_t n, uint32_t root, uint32_t *q0, BfsCtl *ctl,
                                uint32_t max_levels, const uint32_t *outdeg);

namespace {

constexpr int F = bwfeat::COUNT;
constexpr int H = BW_MLP_HIDDEN;
constexpr int OFF_MU = 0, OFF_SD = 12, OFF_W1 = 24, OFF_B1 = OFF_W1 + H * F, OFF_W2 = OFF_B1 + H,
              OFF_B2 = OFF_W2 + H * H, OFF_W3 = OFF_B2 + H;
__host__ __device__ constexpr uint32_t off_b3(uint32_t K) { return OFF_W3 + K * H; }
__host__ __device__ constexpr uint32_t param_count(uint32_t K) { return off_b3(K) + K; }

constexpr int TRAIN_THREADS = 256;
constexpr int MAX_BATCH = 64;

// ------------------------------ MLP kernels --------------------------------
__global__ void k_mlp_init(float *p, uint32_t K, uint64_t seed)
{
    const uint32_t P = param_count(K);
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < P; i += gridDim.x * blockDim.x) {
        if (i < OFF_W1) continue;   // normalisation written by the host
        float fan_in = 0.0f;
        if (i < OFF_B1) fan_in = F;
        else if (i >= OFF_W2 && i < OFF_B2) fan_in = H;
        else if (i >= OFF_W3 && i < off_b3(K)) fan_in = H;
        if (fan_in == 0.0f) { p[i] = 0.0f; continue; }
        // He-uniform: U(-sqrt(6/fan_in), sqrt(6/fan_in)) from the counter hash
        const uint64_t h = bwgen::hash3(seed, i, 99);
        const float u = static_cast<float>(h >> 40) * (1.0f / 16777216.0f);   // [0,1)
        p[i] = (2.0f * u - 1.0f) * sqrtf(6.0f / fan_in);
    }
}

// Forward + backward of one minibatch (sample ids idx[0..B)) into grad
// (accumulated), returns the weighted loss sum (thread 0 valid).
// sp = parameters in shared memory.
__device__ float mlp_batch(const float *sp, uint32_t K, const float *X, const float *T, const float *Wt,
                           const uint32_t *idx, int B, float *sX, float *sH1, float *sH2, float *sZ,
                           float *sG2, float *sG1, float *grad, float *red)
{
    const int tid = threadIdx.x, nt = blockDim.x;
    const float *W1 = sp + OFF_W1, *b1 = sp + OFF_B1, *W2 = sp + OFF_W2, *b2 = sp + OFF_B2;
    const float *W3 = sp + OFF_W3, *b3 = sp + off_b3(K);
    for (int t = tid; t < B * F; t += nt) {
        const int b = t / F, i = t % F;
        const float sd = fmaxf(sp[OFF_SD + i], 1e-6f);
        sX[b * F + i] = (X[static_cast<size_t>(idx[b]) * F + i] - sp[OFF_MU + i]) / sd;
    }
    __syncthreads();
    for (int t = tid; t < B * H; t += nt) {
        const int b = t / H, j = t % H;
        float s = b1[j];
        for (int i = 0; i < F; i++) s += W1[j * F + i] * sX[b * F + i];
        sH1[t] = fmaxf(s, 0.0f);
    }
    __syncthreads();
    for (int t = tid; t < B * H; t += nt) {
        const int b = t / H, j = t % H;
        float s = b2[j];
        for (int i = 0; i < H; i++) s += W2[j * H + i] * sH1[b * H + i];
        sH2[t] = fmaxf(s, 0.0f);
    }
    __syncthreads();
    float loss = 0.0f;
    for (int b = tid; b < B; b += nt) {
        float z[BW_MLP_MAX_CLASSES];
        float mx = -3.0e38f;
        for (uint32_t k = 0; k < K; k++) {
            float s = b3[k];
            for (int i = 0; i < H; i++) s += W3[k * H + i] * sH2[b * H + i];
            z[k] = s;
            mx = fmaxf(mx, s);
        }
        float den = 0.0f;
        for (uint32_t k = 0; k < K; k++) { z[k] = expf(z[k] - mx); den += z[k]; }
        const float w = Wt ? Wt[idx[b]] : 1.0f;
        for (uint32_t k = 0; k < K; k++) {
            const float pk = z[k] / den;
            const float tk = T[static_cast<size_t>(idx[b]) * K + k];
            if (tk > 0.0f) loss -= w * tk * logf(fmaxf(pk, 1e-30f));
            sZ[b * 16 + k] = (pk - tk) * w;      // dL/dz for this sample
        }
    }
    // loss: block reduction into red[0]
    for (int o = 16; o > 0; o >>= 1) loss += __shfl_xor_sync(FULL_MASK, loss, o);
    if ((tid & 31) == 0) red[tid >> 5] = loss;
    __syncthreads();
    float total = 0.0f;
    if (tid == 0)
        for (int w = 0; w < (nt >> 5); w++) total += red[w];
    // dW3, db3
    for (int t = tid; t < static_cast<int>(K) * H; t += nt) {
        const int k = t / H, j = t % H;
        float s = 0.0f;
        for (int b = 0; b < B; b++) s += sZ[b * 16 + k] * sH2[b * H + j];
        grad[OFF_W3 + t] += s;
    }
    for (int k = tid; k < static_cast<int>(K); k += nt) {
        float s = 0.0f;
        for (int b = 0; b < B; b++) s += sZ[b * 16 + k];
        grad[off_b3(K) + k] += s;
    }
    for (int t = tid; t < B * H; t += nt) {
        const int b = t / H, j = t % H;
        float s = 0.0f;
        for (uint32_t k = 0; k < K; k++) s += sZ[b * 16 + k] * W3[k * H + j];
        sG2[t] = sH2[t] > 0.0f ? s : 0.0f;
    }
    __syncthreads();
    for (int t = tid; t < H * H; t += nt) {
        const int o = t / H, i = t % H;
        float s = 0.0f;
        for (int b = 0; b < B; b++) s += sG2[b * H + o] * sH1[b * H + i];
        grad[OFF_W2 + t] += s;
    }
    for (int o = tid; o < H; o += nt) {
        float s = 0.0f;
        for (int b = 0; b < B; b++) s += sG2[b * H + o];
        grad[OFF_B2 + o] += s;
    }
    for (int t = tid; t < B * H; t += nt) {
        const int b = t / H, i = t % H;
        float s = 0.0f;
        for (int o = 0; o < H; o++) s += sG2[b * H + o] * W2[o * H + i];
        sG1[t] = sH1[t] > 0.0f ? s : 0.0f;
    }
    __syncthreads();
    for (int t = tid; t < H * F; t += nt) {
        const int j = t / F, i = t % F;
        float s = 0.0f;
        for (int b = 0; b < B; b++) s += sG1[b * H + j] * sX[b * F + i];
        grad[OFF_W1 + t] += s;
    }
    for (int j = tid; j < H; j += nt) {
        float s = 0.0f;
        for (int b = 0; b < B; b++) s += sG1[b * H + j];
        grad[OFF_B1 + j] += s;
    }
    __syncthreads();
    return total;
}

struct TrainArgs {
    float *params;
    float *adam_m, *adam_v;
    const float *X, *T, *W;
    uint32_t n, K, steps, batch, points;
    float lr, b1, b2, eps, wd;
    uint64_t seed;
    float *loss_curve;   // device [points]
};

// Single-CTA training: every Adam step of the run in one launch.
__global__ void __launch_bounds__(TRAIN_THREADS) k_mlp_train(TrainArgs a)
{
    extern __shared__ float sm[];
    const uint32_t K = a.K, P = param_count(K);
    float *sp = sm;
    float *grad = sp + P;
    float *sX = grad + P;
    float *sH1 = sX + MAX_BATCH * F;
    float *sH2 = sH1 + MAX_BATCH * H;
    float *sG2 = sH2 + MAX_BATCH * H;
    float *sG1 = sG2 + MAX_BATCH * H;
    float *sZ = sG1 + MAX_BATCH * H;
    float *red = sZ + MAX_BATCH * 16;
    uint32_t *idx = reinterpret_cast<uint32_t *>(red + 32);
    const int tid = threadIdx.x, nt = blockDim.x;
    for (uint32_t i = tid; i < P; i += nt) sp[i] = a.params[i];
    __syncthreads();
    float b1t = 1.0f, b2t = 1.0f, loss_acc = 0.0f;
    const uint32_t per_point = a.points ? max(1u, a.steps / a.points) : a.steps + 1;
    const int B = static_cast<int>(min(a.batch, static_cast<uint32_t>(MAX_BATCH)));
    for (uint32_t step = 0; step < a.steps; step++) {
        for (int b = tid; b < B; b += nt) idx[b] = static_cast<uint32_t>(bwgen::bounded(bwgen::hash3(a.seed, step, b), a.n));
        for (uint32_t i = tid; i < P; i += nt) grad[i] = 0.0f;
        __syncthreads();
        const float loss = mlp_batch(sp, K, a.X, a.T, a.W, idx, B, sX, sH1, sH2, sZ, sG2, sG1, grad, red);
        b1t *= a.b1;
        b2t *= a.b2;
        const float inv_b = 1.0f / static_cast<float>(B);
        for (uint32_t i = OFF_W1 + tid; i < P; i += nt) {
            const float g = grad[i] * inv_b + a.wd * sp[i];
            const float m = a.b1 * a.adam_m[i] + (1.0f - a.b1) * g;
            const float v = a.b2 * a.adam_v[i] + (1.0f - a.b2) * g * g;
            a.adam_m[i] = m;
            a.adam_v[i] = v;
            const float mh = m / (1.0f - b1t), vh = v / (1.0f - b2t);
            sp[i] -= a.lr * mh / (sqrtf(vh) + a.eps);
        }
        if (tid == 0) {
            loss_acc += loss * inv_b;
            if (a.points && (step + 1) % per_point == 0) {
                const uint32_t p = (step + 1) / per_point - 1;
                if (p < a.points) a.loss_curve[p] = loss_acc / per_point;
                loss_acc = 0.0f;
            }
        }
        __syncthreads();
    }
    for (uint32_t i = tid; i < P; i += nt) a.params[i] = sp[i];
}

// Full-batch gradient (deterministic order), mean over samples.
__global__ void __launch_bounds__(TRAIN_THREADS) k_mlp_gradient(const float *params, uint32_t K, const float *X,
                                                                const float *T, const float *W, uint32_t n,
                                                                float *grad_out, float *loss_out)
{
    extern __shared__ float sm[];
    const uint32_t P = param_count(K);
    float *sp = sm;
    float *grad = sp + P;
    float *sX = grad + P;
    float *sH1 = sX + MAX_BATCH * F;
    float *sH2 = sH1 + MAX_BATCH * H;
    float *sG2 = sH2 + MAX_BATCH * H;
    float *sG1 = sG2 + MAX_BATCH * H;
    float *sZ = sG1 + MAX_BATCH * H;
    float *red = sZ + MAX_BATCH * 16;
    uint32_t *idx = reinterpret_cast<uint32_t *>(red + 32);
    const int tid = threadIdx.x, nt = blockDim.x;
    for (uint32_t i = tid; i < P; i += nt) { sp[i] = params[i]; grad[i] = 0.0f; }
    __syncthreads();
    float total = 0.0f;
    for (uint32_t base = 0; base < n; base += MAX_BATCH) {
        const int B = static_cast<int>(min(static_cast<uint32_t>(MAX_BATCH), n - base));
        for (int b = tid; b < B; b += nt) idx[b] = base + b;
        __syncthreads();
        total += mlp_batch(sp, K, X, T, W, idx, B, sX, sH1, sH2, sZ, sG2, sG1, grad, red);
    }
    __syncthreads();
    for (uint32_t i = tid; i < P; i += nt) grad_out[i] = i < OFF_W1 ? 0.0f : grad[i] / static_cast<float>(n);
    if (tid == 0) *loss_out = total / static_cast<float>(n);
}

// Thread-per-sample inference.
__device__ __forceinline__ void mlp_forward_one(const float *p, uint32_t K, const float *x_raw, float *probs)
{
    float x[F];
    for (int i = 0; i < F; i++) x[i] = (x_raw[i] - p[OFF_MU + i]) / fmaxf(p[OFF_SD + i], 1e-6f);
    float h1[H];
    for (int j = 0; j < H; j++) {
        float s = p[OFF_B1 + j];
        for (int i = 0; i < F; i++) s += p[OFF_W1 + j * F + i] * x[i];
        h1[j] = fmaxf(s, 0.0f);
    }
    float z[BW_MLP_MAX_CLASSES];
    float h2[H];
    for (int j = 0; j < H; j++) {
        float s = p[OFF_B2 + j];
        for (int i = 0; i < H; i++) s += p[OFF_W2 + j * H + i] * h1[i];
        h2[j] = fmaxf(s, 0.0f);
    }
    float mx = -3.0e38f;
    for (uint32_t k = 0; k < K; k++) {
        float s = p[off_b3(K) + k];
        for (int i = 0; i < H; i++) s += p[OFF_W3 + k * H + i] * h2[i];
        z[k] = s;
        mx = fmaxf(mx, s);
    }
    float den = 0.0f;
    for (uint32_t k = 0; k < K; k++) { z[k] = expf(z[k] - mx); den += z[k]; }
    for (uint32_t k = 0; k < K; k++) probs[k] = z[k] / den;
}

__global__ void k_mlp_predict(const float *params, uint32_t K, const float *X, uint32_t n, float *probs)
{
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x)
        mlp_forward_one(params, K, X + static_cast<size_t>(i) * F, probs + static_cast<size_t>(i) * K);
}

// Host mirror of mlp_forward_one (same operation order).
void mlp_forward_host(const float *p, uint32_t K, const float *x_raw, float *probs)
{
    float x[F];
    for (int i = 0; i < F; i++) x[i] = (x_raw[i] - p[OFF_MU + i]) / std::max(p[OFF_SD + i], 1e-6f);
    float h1[H], h2[H], z[BW_MLP_MAX_CLASSES];
    for (int j = 0; j < H; j++) {
        float s = p[OFF_B1 + j];
        for (int i = 0; i < F; i++) s += p[OFF_W1 + j * F + i] * x[i];
        h1[j] = std::max(s, 0.0f);
    }
    for (int j = 0; j < H; j++) {
        float s = p[OFF_B2 + j];
        for (int i = 0; i < H; i++) s += p[OFF_W2 + j * H + i] * h1[i];
        h2[j] = std::max(s, 0.0f);
    }
    float mx = -3.0e38f;
    for (uint32_t k = 0; k < K; k++) {
        float s = p[off_b3(K) + k];
        for (int i = 0; i < H; i++) s += p[OFF_W3 + k * H + i] * h2[i];
        z[k] = s;
        mx = std::max(mx, s);
    }
    float den = 0.0f;
    for (uint32_t k = 0; k < K; k++) { z[k] = std::exp(z[k] - mx); den += z[k]; }
    for (uint32_t k = 0; k < K; k++) probs[k] = z[k] / den;
}

int pick(const float *probs, uint32_t K, int fallback, float threshold)
{
    int best = 0;
    for (uint32_t k = 1; k < K; k++)
        if (probs[k] > probs[best]) best = static_cast<int>(k);
    return probs[best] < threshold ? fallback : best;
}

size_t train_smem_bytes(uint32_t K)
{
    return (static_cast<size_t>(param_count(K)) * 2 + MAX_BATCH * (F + 4 * H + 16) + 32 + MAX_BATCH) * sizeof(float);
}

// ----------------------- device-side prediction step ----------------------
struct PredictArgs {
    BfsCtl *ctl;
    const float *params;
    uint32_t K;
    int fallback;
    float threshold;
    uint64_t n, m;
    cudaGraphConditionalHandle sw;
    int32_t cluster_k;          // frontier-push's candidate index for cluster-sized frontiers, or -1
};

// Runs before every level inside the device loop: features of the current
// frontier (stats of the previous level, or the root), MLP forward, the
// SWITCH handle for this level's variant.  One block of 128 threads: the
// parameters are staged in shared memory, each thread computes hidden
// units, lane 0 of warp 0 takes the softmax and the decision.
constexpr int PREDICT_THREADS = 128;

__global__ void __launch_bounds__(PREDICT_THREADS) k_bfs_predict(PredictArgs a)
{
    extern __shared__ float sp[];
    __shared__ float x[F], h1[H], h2[H], z[BW_MLP_MAX_CLASSES];
    const int tid = threadIdx.x;
    const uint32_t K = a.K, P = param_count(K);
    for (uint32_t i = tid; i < P; i += PREDICT_THREADS) sp[i] = a.params[i];
    BfsCtl *c = a.ctl;
    const int32_t L = c->depth;
    if (a.cluster_k >= 0) {
        // a frontier the cluster kernel takes goes to frontier-push (the
        // decision is uniform: every thread reads the same slot)
        const LevelSlot s = c->slot[(L + 2) % 3];
        if (s.qlen > 0 && s.qlen <= CLUSTER_CAP && s.fedges <= CLUSTER_EDGE_CAP) {
            if (tid == 0) {
                c->variant = a.cluster_k;
                cudaGraphSetConditional(a.sw, static_cast<unsigned>(a.cluster_k));
            }
            return;
        }
    }
    if (tid == 0) {
        const LevelSlot s = c->slot[(L + 2) % 3];
        float lmax;
        memcpy(&lmax, &s.lmax_bits, 4);
        bwfeat::compute(static_cast<double>(s.frontier), static_cast<double>(s.fedges), lsum_feature(s.lsum),
                        lsq_feature(s.lsq), lmax,
                        static_cast<double>(a.n), static_cast<double>(a.m), static_cast<double>(c->visited),
                        static_cast<double>(c->traversed), static_cast<double>(L), x);
    }
    __syncthreads();
    if (tid < F) x[tid] = (x[tid] - sp[OFF_MU + tid]) / fmaxf(sp[OFF_SD + tid], 1e-6f);
    __syncthreads();
    if (tid < H) {
        float s = sp[OFF_B1 + tid];
        for (int i = 0; i < F; i++) s += sp[OFF_W1 + tid * F + i] * x[i];
        h1[tid] = fmaxf(s, 0.0f);
    }
    __syncthreads();
    if (tid < H) {
        float s = sp[OFF_B2 + tid];
        for (int i = 0; i < H; i++) s += sp[OFF_W2 + tid * H + i] * h1[i];
        h2[tid] = fmaxf(s, 0.0f);
    }
    __syncthreads();
    if (tid < static_cast<int>(K)) {
        float s = sp[off_b3(K) + tid];
        for (int i = 0; i < H; i++) s += sp[OFF_W3 + tid * H + i] * h2[i];
        z[tid] = s;
    }
    __syncthreads();
    if (tid == 0) {
        float mx = -3.0e38f, den = 0.0f;
        for (uint32_t k = 0; k < K; k++) mx = fmaxf(mx, z[k]);
        for (uint32_t k = 0; k < K; k++) den += expf(z[k] - mx);
        int best = 0;
        for (uint32_t k = 1; k < K; k++)
            if (z[k] > z[best]) best = static_cast<int>(k);
        const float pbest = expf(z[best] - mx) / den;
        if (pbest < a.threshold) best = a.fallback;
        c->variant = best;
        cudaGraphSetConditional(a.sw, static_cast<unsigned>(best));
    }
}

__global__ void k_bfs_step_learned(BfsCtl *ctl, LevelSlot *log, uint32_t log_cap, cudaGraphConditionalHandle loop)
{
    if (threadIdx.x != 0 || blockIdx.x != 0) return;
    const int32_t L = ctl->depth;
    LevelSlot s = ctl->slot[L % 3];
    if (log && static_cast<uint32_t>(L) < log_cap) {
        s.heavy = static_cast<uint32_t>(ctl->variant);   // the log keeps the chosen candidate here
        log[L] = s;
    }
    ctl->visited += s.frontier;
    ctl->traversed += s.fedges;
    ctl->levels_done = static_cast<uint32_t>(L) + 1;
    ctl->depth = L + 1;
    ctl->skip = 0;
    bool stop = s.frontier == 0;
    if (!stop && ctl->levels_done >= ctl->max_levels) {
        ctl->status = BW_ERR_LEVEL_LIMIT;
        stop = true;
    }
    if (stop) cudaGraphSetConditional(loop, 0);
}

// Undo a profiled level run: every vertex it visited is in its next-frontier
// queue (parity (L + 1) & 1, length in slot L % 3); reset them to unvisited.
__global__ void k_bfs_undo(int32_t *levels, const BfsCtl *ctl, const uint32_t *q0, const uint32_t *q1, int32_t L)
{
    const uint32_t len = ctl->slot[L % 3].qlen;
    const uint32_t *q = ((L + 1) & 1) ? q1 : q0;
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < len; i += gridDim.x * blockDim.x)
        levels[q[i]] = INF;
}

void slot_stats(const LevelSlot &sl, int variant, bw_bfs_level_stats *out)
{
    out->frontier_vertices = sl.frontier;
    out->variant = static_cast<uint32_t>(variant);
    out->frontier_edges = sl.fedges;
    out->log_degree_sum = static_cast<float>(lsum_value(sl.lsum));
    out->log_degree_sq_sum = static_cast<float>(lsq_value(sl.lsq));
    std::memcpy(&out->log_degree_max, &sl.lmax_bits, 4);
    out->device_ms = 0.0f;
}

struct Plan {
    BfsKernelFn k, k2;
    unsigned block, grid;
    size_t smem;
};

}  // namespace
// Per-block partial log-degree moments of offsets off[0..n]: sum, sum of
// squares and max of log2(1 + degree), written to part[3 * block + 0..2]
// (summed on the host in block order: deterministic).
__global__ void __launch_bounds__(256) k_log_degree_moments(const uint32_t *__restrict__ off, uint64_t n,
                                                            float *__restrict__ part)
{
    __shared__ float r[3][8];
    float ls = 0.f, lq = 0.f, lm = 0.f;
    for (uint64_t v = blockIdx.x * uint64_t(blockDim.x) + threadIdx.x; v < n; v += uint64_t(gridDim.x) * blockDim.x) {
        const float l = __log2f(1.0f + static_cast<float>(off[v + 1] - off[v]));
        ls += l; lq += l * l; lm = fmaxf(lm, l);
    }
    for (int o = 16; o > 0; o >>= 1) {
        ls += __shfl_xor_sync(FULL_MASK, ls, o);
        lq += __shfl_xor_sync(FULL_MASK, lq, o);
        lm = fmaxf(lm, __shfl_xor_sync(FULL_MASK, lm, o));
    }
    const unsigned w = threadIdx.x >> 5, lane = threadIdx.x & 31;
    if (lane == 0) { r[0][w] = ls; r[1][w] = lq; r[2][w] = lm; }
    __syncthreads();
    if (threadIdx.x == 0) {
        float a = 0.f, b = 0.f, c = 0.f;
        for (unsigned i = 0; i < blockDim.x / 32; i++) { a += r[0][i]; b += r[1][i]; c = fmaxf(c, r[2][i]); }
        part[3 * blockIdx.x] = a;
        part[3 * blockIdx.x + 1] = b;
        part[3 * blockIdx.x + 2] = c;
    }
}

// The log-degree moments of the view's in-degrees (out-degrees when it has
// no reverse CSR): block partials summed on the host in block order.
int pagerank_moments(bw_context *ctx, const bw_graph_view *g, float *ls, float *lq, float *lm, cudaStream_t s)
{
    if (!ctx || !g || g->vertex_count == 0 || g->vertex_count > 0xffffffffULL) return BW_ERR_INVALID_ARGUMENT;
    const uint32_t *off = g->rev_vertices ? g->rev_vertices : g->fwd_vertices;
    if (!off) return BW_ERR_MISSING_REPRESENTATION;
    const unsigned blocks = static_cast<unsigned>(ctx->sm_count) * 2u;
    float *part = nullptr;
    BW_CUDA(ctx_malloc_async(ctx, reinterpret_cast<void **>(&part), blocks * 3 * sizeof(float), s));
    k_log_degree_moments<<<blocks, 256, 0, s>>>(off, g->vertex_count, part);
    const cudaError_t e = cudaGetLastError();
    std::vector<float> h(blocks * 3);
    if (e == cudaSuccess) cudaMemcpyAsync(h.data(), part, h.size() * sizeof(float), cudaMemcpyDeviceToHost, s);
    cudaFreeAsync(part, s);
    BW_CUDA(e);
    BW_CUDA(cudaStreamSynchronize(s));
    *ls = *lq = *lm = 0.f;
    for (unsigned b = 0; b < blocks; b++) { *ls += h[3 * b]; *lq += h[3 * b + 1]; *lm = std::max(*lm, h[3 * b + 2]); }
    return BW_OK;
}

// A PageRank iteration's features: every vertex is active, so the whole
// vertex set is the frontier and nothing is left unvisited.  The level
// separates the first iteration (0) from the rest (1): after the first, an
// iteration does the same work every time.
void pagerank_feature_vector(const bw_graph_view *g, float ls, float lq, float lm, uint32_t iteration, float *x)
{
    const double n = static_cast<double>(g->vertex_count), m = static_cast<double>(g->edge_count);
    bwfeat::compute(n, m, ls, lq, lm, n, m, n, m, iteration == 0 ? 0.0 : 1.0, x);
}

// The frontier {root} before level 0, with the statistics the level kernels
// accumulate (the same formula as the side-statistics initialisation).
__global__ void k_bfs_root_stats(const uint32_t *outdeg, uint32_t root, LevelSlot *out)
{
    if (blockIdx.x == 0 && threadIdx.x == 0) {
        const uint32_t d = outdeg[root];
        const float l = __log2f(1.0f + static_cast<float>(d));
        *out = LevelSlot{};
        out->frontier = 1;
        out->qlen = 1;
        out->fedges = d;
        out->lsum = lsum_fx(l);
        out->lsq = lsq_fx(l);
        out->lmax_bits = __float_as_uint(l);
    }
}

}  // namespace bw

using namespace bw;

extern "C" {

uint32_t bw_mlp_param_count(uint32_t classes) { return param_count(classes); }

void bw_bfs_features(uint64_t fv, uint64_t fe, float lsum, float lsq, float lmax, uint64_t n, uint64_t m,
                     uint64_t visited, uint64_t edges_visited, uint32_t level, float out[12])
{
    bwfeat::compute(static_cast<double>(fv), static_cast<double>(fe), lsum, lsq, lmax, static_cast<double>(n),
                    static_cast<double>(m), static_cast<double>(visited), static_cast<double>(edges_visited),
                    static_cast<double>(level), out);
}

int bw_mlp_predict_host(const float *params, uint32_t classes, const float *features, uint32_t n, float *probs)
{
    if (!params || !features || !probs || classes < 2 || classes > BW_MLP_MAX_CLASSES) return BW_ERR_INVALID_ARGUMENT;
    for (uint32_t i = 0; i < n; i++)
        mlp_forward_host(params, classes, features + static_cast<size_t>(i) * F, probs + static_cast<size_t>(i) * classes);
    return BW_OK;
}

int bw_pagerank_features(bw_context *ctx, const bw_graph_view *g, uint32_t iteration, float out[12], void *stream)
{
    if (!out) return BW_ERR_INVALID_ARGUMENT;
    float ls = 0.f, lq = 0.f, lm = 0.f;
    BW_TRY(pagerank_moments(ctx, g, &ls, &lq, &lm, as_stream(stream)));
    pagerank_feature_vector(g, ls, lq, lm, iteration, out);
    return BW_OK;
}

int bw_pagerank_run_learned(bw_context *ctx, const bw_graph_view *g, const bw_switch_config *sw,
                            uint32_t iterations, float *ranks, int loop_mode, bw_pagerank_result *result,
                            float *diffs, int32_t *schedule_out, void *stream)
{
    if (!ctx || !g || !sw || !sw->params || !sw->candidates || sw->classes < 2 || sw->classes > BW_MLP_MAX_CLASSES)
        return BW_ERR_INVALID_ARGUMENT;
    const uint32_t K = sw->classes;
    if (sw->fallback < 0 || static_cast<uint32_t>(sw->fallback) >= K) return BW_ERR_INVALID_ARGUMENT;
    cudaStream_t s = as_stream(stream);
    std::vector<float> hp(param_count(K));
    BW_CUDA(cudaMemcpyAsync(hp.data(), sw->params, hp.size() * sizeof(float), cudaMemcpyDeviceToHost, s));
    float ls = 0.f, lq = 0.f, lm = 0.f;
    // also completes the parameter copy (it synchronises the stream)
    if (const int rc = pagerank_moments(ctx, g, &ls, &lq, &lm, s); rc != BW_OK) {
        cudaStreamSynchronize(s);        // hp must outlive the copy
        return rc;
    }
    // The features depend on the iteration index only, so the whole
    // schedule is chosen before the run; they take two values (the first
    // iteration, every later one), so the network runs twice.
    std::vector<int32_t> sched(std::max<uint32_t>(iterations, 1u));
    int32_t choice[2];
    for (uint32_t it = 0; it < 2; it++) {
        float x[F], probs[BW_MLP_MAX_CLASSES];
        pagerank_feature_vector(g, ls, lq, lm, it, x);
        mlp_forward_host(hp.data(), K, x, probs);
        choice[it] = sw->candidates[pick(probs, K, sw->fallback, sw->threshold)];
    }
    for (uint32_t it = 0; it < sched.size(); it++) sched[it] = choice[it ? 1 : 0];
    if (schedule_out)
        for (uint32_t it = 0; it < iterations; it++) schedule_out[it] = sched[it];
    return pagerank_run_schedule_loop(ctx, g, sched.data(), static_cast<uint32_t>(sched.size()), iterations, ranks,
                                      loop_mode, result, diffs, s);
}

int bw_bfs_frontier_stats(bw_context *ctx, const bw_graph_view *g, uint32_t root, int32_t depth,
                          bw_bfs_level_stats *out, void *stream)
{
    if (!ctx || !g || !out) return BW_ERR_INVALID_ARGUMENT;
    if (!g->fwd_vertices) return BW_ERR_MISSING_REPRESENTATION;
    cudaStream_t s = as_stream(stream);
    LevelSlot sl{};
    if (depth < 0) {
        if (root >= g->vertex_count) return BW_ERR_INVALID_ARGUMENT;
        BW_TRY(ensure_outdeg(ctx, g, s));
        LevelSlot *d = nullptr;
        BW_CUDA(ctx_malloc_async(ctx, reinterpret_cast<void **>(&d), sizeof(LevelSlot), s));
        k_bfs_root_stats<<<1, 32, 0, s>>>(ctx->outdeg, root, d);
        const cudaError_t e = cudaGetLastError();
        if (e == cudaSuccess) cudaMemcpyAsync(&sl, d, sizeof(LevelSlot), cudaMemcpyDeviceToHost, s);
        cudaFreeAsync(d, s);
        BW_CUDA(e);
    } else {
        // bw_bfs_level at this depth left its counts in slot depth % 3
        if (!ctx->bfs_ctl) return BW_ERR_INVALID_ARGUMENT;
        BW_CUDA(cudaMemcpyAsync(&sl, &ctx->bfs_ctl->slot[depth % 3], sizeof(LevelSlot), cudaMemcpyDeviceToHost, s));
    }
    BW_CUDA(cudaStreamSynchronize(s));
    slot_stats(sl, -1, out);
    return BW_OK;
}

int bw_mlp_init(float *params, uint32_t classes, const float *mu, const float *sd, uint64_t seed, void *stream)
{
    if (!params || !mu || !sd || classes < 2 || classes > BW_MLP_MAX_CLASSES) return BW_ERR_INVALID_ARGUMENT;
    cudaStream_t s = as_stream(stream);
    k_mlp_init<<<16, 256, 0, s>>>(params, classes, seed);
    BW_CUDA(cudaGetLastError());
    BW_CUDA(cudaMemcpyAsync(params + OFF_MU, mu, F * sizeof(float), cudaMemcpyHostToDevice, s));
    BW_CUDA(cudaMemcpyAsync(params + OFF_SD, sd, F * sizeof(float), cudaMemcpyHostToDevice, s));
    BW_CUDA(cudaStreamSynchronize(s));
    return BW_OK;
}

int bw_mlp_train(bw_context *ctx, float *params, uint32_t classes, const float *X, const float *T, const float *W,
                 uint32_t n, const bw_mlp_train_config *cfg, float *loss_curve, uint32_t loss_points, void *stream)
{
    if (!ctx || !params || !X || !T || !cfg || n == 0 || classes < 2 || classes > BW_MLP_MAX_CLASSES)
        return BW_ERR_INVALID_ARGUMENT;
    if (cfg->batch == 0 || cfg->batch > MAX_BATCH) return BW_ERR_INVALID_ARGUMENT;
    cudaStream_t s = as_stream(stream);
    const uint32_t P = param_count(classes);
    TrainArgs a{};
    a.params = params; a.X = X; a.T = T; a.W = W; a.n = n; a.K = classes;
    a.steps = cfg->steps; a.batch = cfg->batch; a.lr = cfg->lr; a.b1 = cfg->beta1; a.b2 = cfg->beta2;
    a.eps = cfg->eps; a.wd = cfg->weight_decay; a.seed = cfg->seed; a.points = loss_curve ? loss_points : 0;
    float *scratch = nullptr;
    BW_CUDA(ctx_malloc_async(ctx, reinterpret_cast<void **>(&scratch), (2 * P + a.points + 1) * sizeof(float), s));
    BW_CUDA(cudaMemsetAsync(scratch, 0, (2 * P + a.points + 1) * sizeof(float), s));
    a.adam_m = scratch; a.adam_v = scratch + P; a.loss_curve = scratch + 2 * P;
    const size_t smem = train_smem_bytes(classes);
    BW_CUDA(cudaFuncSetAttribute(k_mlp_train, cudaFuncAttributeMaxDynamicSharedMemorySize, static_cast<int>(smem)));
    k_mlp_train<<<1, TRAIN_THREADS, smem, s>>>(a);
    BW_CUDA(cudaGetLastError());
    if (a.points) BW_CUDA(cudaMemcpyAsync(loss_curve, a.loss_curve, a.points * sizeof(float), cudaMemcpyDeviceToHost, s));
    BW_CUDA(cudaFreeAsync(scratch, s));
    BW_CUDA(cudaStreamSynchronize(s));
    return BW_OK;
}

int bw_mlp_gradient(bw_context *ctx, const float *params, uint32_t classes, const float *X, const float *T,
                    const float *W, uint32_t n, float *grad, float *loss, void *stream)
{
    if (!ctx || !params || !X || !T || !grad || n == 0 || classes < 2 || classes > BW_MLP_MAX_CLASSES)
        return BW_ERR_INVALID_ARGUMENT;
    cudaStream_t s = as_stream(stream);
    float *dloss = nullptr;
    BW_CUDA(ctx_malloc_async(ctx, reinterpret_cast<void **>(&dloss), sizeof(float), s));
    const size_t smem = train_smem_bytes(classes);
    BW_CUDA(cudaFuncSetAttribute(k_mlp_gradient, cudaFuncAttributeMaxDynamicSharedMemorySize, static_cast<int>(smem)));
    k_mlp_gradient<<<1, TRAIN_THREADS, smem, s>>>(params, classes, X, T, W, n, grad, dloss);
    BW_CUDA(cudaGetLastError());
    float h = 0.0f;
    BW_CUDA(cudaMemcpyAsync(&h, dloss, sizeof h, cudaMemcpyDeviceToHost, s));
    BW_CUDA(cudaFreeAsync(dloss, s));
    BW_CUDA(cudaStreamSynchronize(s));
    if (loss) *loss = h;
    return BW_OK;
}

int bw_mlp_predict(bw_context *ctx, const float *params, uint32_t classes, const float *X, uint32_t n,
                   float *probs, void *stream)
{
    if (!ctx || !params || !X || !probs || classes < 2 || classes > BW_MLP_MAX_CLASSES) return BW_ERR_INVALID_ARGUMENT;
    if (n == 0) return BW_OK;
    k_mlp_predict<<<(n + 127) / 128, 128, 0, as_stream(stream)>>>(params, classes, X, n, probs);
    BW_CUDA(cudaGetLastError());
    return BW_OK;
}

int bw_bfs_profile(bw_context *ctx, const bw_graph_view *g, uint32_t root, int32_t *levels,
                   const int32_t *candidates, uint32_t K, uint32_t max_levels, uint32_t repeats,
                   uint32_t sample_every, uint32_t default_index, float *level_ms, float *features,
                   uint32_t *level_count, void *stream)
{
    if (!candidates || K == 0 || !level_ms || !features || max_levels == 0 || default_index >= K)
        return BW_ERR_INVALID_ARGUMENT;
    cudaStream_t s = as_stream(stream);
    int reps = 1;
    for (uint32_t k = 0; k < K; k++) {
        if (bfs_variant_reps(candidates[k]) == 0) return BW_ERR_UNKNOWN_VARIANT;
        reps |= bfs_variant_reps(candidates[k]);
    }
    BW_TRY(bfs_prepare(ctx, g, reps, true, levels, root, s));
    std::vector<Plan> plans(K);
    for (uint32_t k = 0; k < K; k++)
        BW_TRY(bfs_plan(ctx, candidates[k], true, nullptr, &plans[k].k, &plans[k].k2, &plans[k].block,
                        &plans[k].grid, &plans[k].smem));
    if (repeats == 0) repeats = 1;
    if (sample_every == 0) sample_every = 1;
    const uint64_t n = g->vertex_count, m = g->edge_count;
    BfsCtl *ctl_snap = nullptr;
    BW_CUDA(ctx_malloc_async(ctx, reinterpret_cast<void **>(&ctl_snap), sizeof(BfsCtl), s));
    BW_TRY(ensure_level_events(ctx, 2));
    k_bfs_init_side<<<ctx->sm_count * 4, 256, 0, s>>>(levels, n, root, ctx->queue[0], ctx->bfs_ctl, max_levels,
                                                     ctx->outdeg);
    BW_CUDA(cudaGetLastError());
    BW_CUDA(cudaMemcpyAsync(ctx->bfs_ctl_host, ctx->bfs_ctl, sizeof(BfsCtl), cudaMemcpyDeviceToHost, s));
    BW_CUDA(cudaStreamSynchronize(s));
    LevelSlot cur = ctx->bfs_ctl_host->slot[2];     // the root as frontier
    uint64_t visited = 1, edges_visited = cur.fedges;
    uint32_t L = 0;
    int rc = BW_OK;
    std::vector<float> times(repeats);
    auto run_one = [&](uint32_t k) {
        BfsArgs a = bfs_args(ctx, g, levels, static_cast<int32_t>(L), nullptr);
        plans[k].k<<<plans[k].grid, plans[k].block, plans[k].smem, s>>>(a);
        if (plans[k].k2) plans[k].k2<<<hub_grid(plans[k].grid, plans[k].block), 256, 0, s>>>(a);
    };
    for (; L < max_levels; L++) {
        float lmax;
        std::memcpy(&lmax, &cur.lmax_bits, 4);
        bwfeat::compute(cur.frontier, static_cast<double>(cur.fedges), lsum_feature(cur.lsum), lsq_feature(cur.lsq), lmax,
                        static_cast<double>(n),
                        static_cast<double>(m), static_cast<double>(visited), static_cast<double>(edges_visited), L,
                        features + static_cast<size_t>(L) * F);
        const bool sampled = L < 32 || L % sample_every == 0;
        if (sampled) {
            BW_CUDA(cudaMemcpyAsync(ctl_snap, ctx->bfs_ctl, sizeof(BfsCtl), cudaMemcpyDeviceToDevice, s));
            for (uint32_t k = 0; k < K; k++) {
                for (uint32_t r = 0; r < repeats; r++) {
                    const bool last = k + 1 == K && r + 1 == repeats;
                    BW_CUDA(cudaEventRecord(ctx->level_events[0], s));
                    run_one(k);
                    BW_CUDA(cudaEventRecord(ctx->level_events[1], s));
                    BW_CUDA(cudaGetLastError());
                    if (!last) {
                        // undo: the vertices this run visited are in its queue
                        k_bfs_undo<<<ctx->sm_count * 2, 256, 0, s>>>(levels, ctx->bfs_ctl, ctx->queue[0],
                                                                      ctx->queue[1], static_cast<int32_t>(L));
                        BW_CUDA(cudaMemcpyAsync(ctx->bfs_ctl, ctl_snap, sizeof(BfsCtl), cudaMemcpyDeviceToDevice, s));
                    }
                    BW_CUDA(cudaEventSynchronize(ctx->level_events[1]));
                    BW_CUDA(cudaEventElapsedTime(&times[r], ctx->level_events[0], ctx->level_events[1]));
                }
                std::sort(times.begin(), times.end());
                level_ms[static_cast<size_t>(L) * K + k] = times[repeats / 2];
            }
        } else {
            run_one(default_index);
            BW_CUDA(cudaGetLastError());
            for (uint32_t k = 0; k < K; k++) level_ms[static_cast<size_t>(L) * K + k] = -1.0f;
        }
        BW_CUDA(cudaMemcpyAsync(&ctx->bfs_ctl_host->slot[L % 3], &ctx->bfs_ctl->slot[L % 3], sizeof(LevelSlot),
                                cudaMemcpyDeviceToHost, s));
        BW_CUDA(cudaStreamSynchronize(s));
        cur = ctx->bfs_ctl_host->slot[L % 3];
        visited += cur.frontier;
        edges_visited += cur.fedges;
        if (cur.frontier == 0) { L++; break; }
    }
    if (L >= max_levels && cur.frontier != 0) rc = BW_ERR_LEVEL_LIMIT;
    cudaFreeAsync(ctl_snap, s);
    BW_CUDA(cudaStreamSynchronize(s));
    if (level_count) *level_count = L;
    return rc;
}

int bw_bfs_run_learned(bw_context *ctx, const bw_graph_view *g, const bw_switch_config *sw, uint32_t root,
                       int32_t *levels, int loop_mode, uint32_t max_levels, bw_bfs_result *result,
                       bw_bfs_level_stats *stats, uint32_t stats_cap, void *stream)
{
    if (!sw || !sw->params || !sw->candidates || sw->classes < 2 || sw->classes > BW_MLP_MAX_CLASSES)
        return BW_ERR_INVALID_ARGUMENT;
    const uint32_t K = sw->classes;
    if (sw->fallback < 0 || static_cast<uint32_t>(sw->fallback) >= K) return BW_ERR_INVALID_ARGUMENT;
    cudaStream_t s = as_stream(stream);
    if (loop_mode != BW_LOOP_GRAPH && loop_mode != BW_LOOP_HOST) return BW_ERR_INVALID_ARGUMENT;
    if (g && g->edge_count == 0)      // no level kernel runs: nothing to choose
        return bfs_edgeless(ctx, g, sw->candidates[sw->fallback], root, levels, result, stats, stats_cap, s);
    int reps = 1;
    for (uint32_t k = 0; k < K; k++) {
        if (bfs_variant_reps(sw->candidates[k]) == 0) return BW_ERR_UNKNOWN_VARIANT;
        reps |= bfs_variant_reps(sw->candidates[k]);
    }
    BW_TRY(bfs_prepare(ctx, g, reps, true, levels, root, s));
    std::vector<Plan> plans(K);
    for (uint32_t k = 0; k < K; k++)
        BW_TRY(bfs_plan(ctx, sw->candidates[k], true, nullptr, &plans[k].k, &plans[k].k2, &plans[k].block,
                        &plans[k].grid, &plans[k].smem));
    const uint64_t n = g->vertex_count, m = g->edge_count;
    if (max_levels == 0) max_levels = static_cast<uint32_t>(std::min<uint64_t>(n + 1, 0xffffffffULL));

    if (loop_mode == BW_LOOP_HOST) {
        std::vector<float> hp(param_count(K));
        BW_CUDA(cudaMemcpyAsync(hp.data(), sw->params, hp.size() * sizeof(float), cudaMemcpyDeviceToHost, s));
        k_bfs_init_side<<<ctx->sm_count * 4, 256, 0, s>>>(levels, n, root, ctx->queue[0], ctx->bfs_ctl, max_levels,
                                                         ctx->outdeg);
        BW_CUDA(cudaMemcpyAsync(ctx->bfs_ctl_host, ctx->bfs_ctl, sizeof(BfsCtl), cudaMemcpyDeviceToHost, s));
        BW_CUDA(cudaStreamSynchronize(s));
        LevelSlot cur = ctx->bfs_ctl_host->slot[2];
        uint64_t visited = 1, edges_visited = cur.fedges;
        BW_CUDA(cudaEventRecord(ctx->ev_start, s));
        uint32_t L = 0;
        int rc = BW_OK;
        for (;;) {
            if (L >= max_levels) { rc = BW_ERR_LEVEL_LIMIT; break; }
            float x[F], probs[BW_MLP_MAX_CLASSES], lmax;
            std::memcpy(&lmax, &cur.lmax_bits, 4);
            bwfeat::compute(cur.frontier, static_cast<double>(cur.fedges), lsum_feature(cur.lsum), lsq_feature(cur.lsq), lmax,
                            static_cast<double>(n), static_cast<double>(m), static_cast<double>(visited),
                            static_cast<double>(edges_visited), L, x);
            mlp_forward_host(hp.data(), K, x, probs);
            const int c = pick(probs, K, sw->fallback, sw->threshold);
            BfsArgs a = bfs_args(ctx, g, levels, static_cast<int32_t>(L), nullptr);
            plans[c].k<<<plans[c].grid, plans[c].block, plans[c].smem, s>>>(a);
            if (plans[c].k2) plans[c].k2<<<hub_grid(plans[c].grid, plans[c].block), 256, 0, s>>>(a);
            BW_CUDA(cudaGetLastError());
            BW_CUDA(cudaMemcpyAsync(&ctx->bfs_ctl_host->slot[L % 3], &ctx->bfs_ctl->slot[L % 3], sizeof(LevelSlot),
                                    cudaMemcpyDeviceToHost, s));
            BW_CUDA(cudaStreamSynchronize(s));
            cur = ctx->bfs_ctl_host->slot[L % 3];
            if (stats && L < stats_cap) slot_stats(cur, sw->candidates[c], &stats[L]);
            visited += cur.frontier;
            edges_visited += cur.fedges;
            L++;
            if (cur.frontier == 0) break;
        }
        BW_CUDA(cudaEventRecord(ctx->ev_stop, s));
        BW_CUDA(cudaEventSynchronize(ctx->ev_stop));
        if (result) {
            float ms = 0.0f;
            BW_CUDA(cudaEventElapsedTime(&ms, ctx->ev_start, ctx->ev_stop));
            result->level_count = L;
            result->visited = visited;
            result->device_ms = ms;
            BW_TRY(bfs_traversed(ctx, g, levels, s, &result->traversed_edges));
        }
        return rc;
    }
    if (loop_mode != BW_LOOP_GRAPH) return BW_ERR_INVALID_ARGUMENT;

    // Device loop: WHILE { predict -> SWITCH(K level bodies) -> step }.
    BW_TRY(bfs_cluster_prepare());          // frontier-push's small-frontier kernel, if a candidate
    LevelSlot *log = nullptr;
    const uint32_t log_cap = stats ? std::min(stats_cap, max_levels) : 0;
    if (log_cap) BW_CUDA(ctx_malloc_async(ctx, reinterpret_cast<void **>(&log), log_cap * sizeof(LevelSlot), s));
    cudaGraph_t graph = nullptr;
    cudaGraphExec_t exec = nullptr;
    int rc = BW_OK;
    auto fail = [&](cudaError_t e, const char *what) {
        set_last_error(e, what);
        rc = e == cudaErrorMemoryAllocation ? BW_ERR_OUT_OF_MEMORY : BW_ERR_CUDA;
    };
    do {
        cudaError_t e = cudaGraphCreate(&graph, 0);
        if (e != cudaSuccess) { fail(e, "cudaGraphCreate"); break; }
        cudaGraphConditionalHandle loop;
        if ((e = cudaGraphConditionalHandleCreate(&loop, graph, 1, cudaGraphCondAssignDefault)) != cudaSuccess) {
            fail(e, "handle(loop)"); break;
        }
        cudaGraphNodeParams wp = {};
        wp.type = cudaGraphNodeTypeConditional;
        wp.conditional.handle = loop;
        wp.conditional.type = cudaGraphCondTypeWhile;
        wp.conditional.size = 1;
        cudaGraphNode_t wnode;
        if ((e = cudaGraphAddNode(&wnode, graph, nullptr, nullptr, 0, &wp)) != cudaSuccess) { fail(e, "while node"); break; }
        cudaGraph_t body = wp.conditional.phGraph_out[0];
        cudaGraphConditionalHandle swh;
        if ((e = cudaGraphConditionalHandleCreate(&swh, body, 0, cudaGraphCondAssignDefault)) != cudaSuccess) {
            fail(e, "handle(switch)"); break;
        }
        // predict kernel node
        int32_t cluster_k = -1;
        if (!(sw->flags & BW_SWITCH_MLP_ONLY))
            for (uint32_t k = 0; k < K; k++)
                if (sw->candidates[k] == 32) cluster_k = static_cast<int32_t>(k);   // frontier-push
        PredictArgs pa{ctx->bfs_ctl, sw->params, K, sw->fallback, sw->threshold, n, m, swh, cluster_k};
        cudaKernelNodeParams kp = {};
        void *pargs[] = {&pa};
        kp.func = reinterpret_cast<void *>(k_bfs_predict);
        kp.gridDim = dim3(1);
        kp.blockDim = dim3(PREDICT_THREADS);
        kp.sharedMemBytes = param_count(K) * sizeof(float);
        kp.kernelParams = pargs;
        cudaGraphNode_t pnode;
        if ((e = cudaGraphAddKernelNode(&pnode, body, nullptr, 0, &kp)) != cudaSuccess) { fail(e, "predict node"); break; }
        cudaGraphNodeParams sp = {};
        sp.type = cudaGraphNodeTypeConditional;
        sp.conditional.handle = swh;
        sp.conditional.type = cudaGraphCondTypeSwitch;
        sp.conditional.size = K;
        cudaGraphNode_t snode;
        if ((e = cudaGraphAddNode(&snode, body, &pnode, nullptr, 1, &sp)) != cudaSuccess) { fail(e, "switch node"); break; }
        BfsArgs a = bfs_args(ctx, g, levels, -1, nullptr);
        a.skip_check = 1;
        a.log = log;
        a.log_cap = log_cap;
        for (uint32_t k = 0; k < K && rc == BW_OK; k++) {
            cudaGraph_t kb = sp.conditional.phGraph_out[k];
            void *kargs[] = {&a};
            cudaGraphNode_t first = nullptr;
            if (sw->candidates[k] == 32) {      // frontier-push: small-frontier cluster path first
                cudaKernelNodeParams cp = {};
                // the level log needs every level's statistics; otherwise
                // only a handed-over level's, which the next prediction reads
                cp.func = reinterpret_cast<void *>(bfs_cluster_kernel(log_cap ? 1 : 2));
                cp.gridDim = dim3(CLUSTER_CTAS);
                cp.blockDim = dim3(CLUSTER_THREADS);
                cp.sharedMemBytes = static_cast<unsigned>(bfs_cluster_smem());
                cp.kernelParams = kargs;
                if ((e = cudaGraphAddKernelNode(&first, kb, nullptr, 0, &cp)) != cudaSuccess) { fail(e, "cluster node"); break; }
            }
            cudaKernelNodeParams lp = {};
            lp.func = reinterpret_cast<void *>(plans[k].k);
            lp.gridDim = dim3(plans[k].grid);
            lp.blockDim = dim3(plans[k].block);
            lp.sharedMemBytes = static_cast<unsigned>(plans[k].smem);
            lp.kernelParams = kargs;
            cudaGraphNode_t n1;
            if ((e = cudaGraphAddKernelNode(&n1, kb, first ? &first : nullptr, first ? 1 : 0, &lp)) != cudaSuccess) {
                fail(e, "level node"); break;
            }
            if (plans[k].k2) {
                cudaKernelNodeParams lp2 = lp;
                lp2.func = reinterpret_cast<void *>(plans[k].k2);
                lp2.gridDim = dim3(hub_grid(plans[k].grid, plans[k].block));
                lp2.blockDim = dim3(256);
                lp2.sharedMemBytes = 0;
                cudaGraphNode_t n2;
                if ((e = cudaGraphAddKernelNode(&n2, kb, &n1, 1, &lp2)) != cudaSuccess) { fail(e, "hub node"); break; }
            }
        }
        if (rc) break;
        LevelSlot *logp = log;
        uint32_t lc = log_cap;
        BfsCtl *ctlp = ctx->bfs_ctl;
        void *sargs[] = {&ctlp, &logp, &lc, &loop};
        cudaKernelNodeParams stp = {};
        stp.func = reinterpret_cast<void *>(k_bfs_step_learned);
        stp.gridDim = dim3(1);
        stp.blockDim = dim3(32);
        stp.kernelParams = sargs;
        cudaGraphNode_t stnode;
        if ((e = cudaGraphAddKernelNode(&stnode, body, &snode, 1, &stp)) != cudaSuccess) { fail(e, "step node"); break; }
        if ((e = cudaGraphInstantiate(&exec, graph, 0)) != cudaSuccess) { fail(e, "instantiate"); break; }
    } while (0);
    if (rc) {
        if (graph) cudaGraphDestroy(graph);
        if (log) cudaFreeAsync(log, s);
        return rc;
    }
    k_bfs_init_side<<<ctx->sm_count * 4, 256, 0, s>>>(levels, n, root, ctx->queue[0], ctx->bfs_ctl, max_levels,
                                                     ctx->outdeg);
    BW_CUDA(cudaGetLastError());
    BW_CUDA(cudaEventRecord(ctx->ev_start, s));
    BW_CUDA(cudaGraphLaunch(exec, s));
    BW_CUDA(cudaEventRecord(ctx->ev_stop, s));
    BW_CUDA(cudaMemcpyAsync(ctx->bfs_ctl_host, ctx->bfs_ctl, sizeof(BfsCtl), cudaMemcpyDeviceToHost, s));
    BW_CUDA(cudaStreamSynchronize(s));
    cudaGraphExecDestroy(exec);
    cudaGraphDestroy(graph);
    const BfsCtl c = *ctx->bfs_ctl_host;
    if (log_cap) {
        const uint32_t got = std::min(c.levels_done, log_cap);
        std::vector<LevelSlot> tmp(got ? got : 1);
        BW_CUDA(cudaMemcpy(tmp.data(), log, got * sizeof(LevelSlot), cudaMemcpyDeviceToHost));
        for (uint32_t i = 0; i < got; i++) slot_stats(tmp[i], sw->candidates[tmp[i].heavy], &stats[i]);
        BW_CUDA(cudaFreeAsync(log, s));
    }
    if (result) {
        float ms = 0.0f;
        BW_CUDA(cudaEventElapsedTime(&ms, ctx->ev_start, ctx->ev_stop));
        result->level_count = c.levels_done;
        result->visited = c.visited;
        result->device_ms = ms;
        BW_TRY(bfs_traversed(ctx, g, levels, s, &result->traversed_edges));
    }
    return c.status ? static_cast<int>(c.status) : BW_OK;
}

}  // extern "C"
