/*
 * Learned cost model for the autotuner (no reference counterpart: GPUfs has
 * no tuner).  A small fully connected network, n_in -> 64 -> 64 -> 1 with
 * tanh hidden units in FP32, predicts a run's log time from workload
 * features (file-size histogram, op mix, file count, bytes) and session
 * parameters (page size, host workers, grid, staging depth).  It never sees
 * file bytes, so the data path stays exact.
 *
 * Training is two kernels per step, both deterministic:
 *   k_cm_pass<true>  each CTA runs forward and backward over 32-sample tiles
 *                    (tile t goes to CTA t mod grid), keeps its weight
 *                    gradients in registers, and writes one partial
 *                    gradient row;
 *   k_cm_reduce      sums the rows in CTA order per parameter, then takes
 *                    an Adam step (or hands the gradient back, for checks).
 * Loss: mean squared error over the data set.  Parameters, one flat FP32
 * vector: W1 [n_in][64], b1 [64], W2 [64][64], b2 [64], w3 [64], b3.
 */
#include <cuda_runtime.h>
#include <math.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>

#include <vector>

#include "gfs_types.h"
#include "gpufs_gb300.h"

namespace {

constexpr int H = GFS_CM_HIDDEN; /* hidden width */
constexpr int DMAX = GFS_CM_MAX_INPUTS;
constexpr int TS = 32;           /* samples per tile */
constexpr int NT = 256;          /* threads per CTA: 64 columns x 4 row groups */
constexpr int MAX_CTAS = 152;
constexpr int GRAPH_STEPS = 32;  /* training steps per captured graph */
static_assert(H == 64 && NT == 256, "thread mapping assumes 64 columns x 4 row groups");

struct Lay {
    int d, w1, b1, w2, b2, w3, b3, p;
};
__host__ __device__ inline Lay lay(int d) {
    Lay L;
    L.d = d;
    L.w1 = 0;
    L.b1 = d * H;
    L.w2 = L.b1 + H;
    L.b2 = L.w2 + H * H;
    L.w3 = L.b2 + H;
    L.b3 = L.w3 + H;
    L.p = L.b3 + 1;
    return L;
}

/* shared floats of one CTA */
inline size_t smem_floats(int d) { return (size_t)d * H + 3 * H + H * H + (size_t)TS * d + 4 * TS * H + TS + 3 * 4 * H + 8; }

/* One pass over the data set.  BWD: forward + backward, partial gradient
 * rows into part[blockIdx.x][P] and partial losses into lossp; otherwise
 * forward only, predictions into y_out.  step: incremented once per
 * training pass (read by the Adam step that follows). */
template <bool BWD>
__global__ void __launch_bounds__(NT) k_cm_pass(const float* __restrict__ params, const float* __restrict__ X,
                                                const float* __restrict__ tgt, int n, int d, float* __restrict__ part,
                                                float* __restrict__ lossp, float* __restrict__ y_out, int* step) {
    extern __shared__ float sm[];
    const Lay L = lay(d);
    float* w1 = sm;
    float* b1 = w1 + d * H;
    float* w2 = b1 + H;
    float* b2 = w2 + H * H;
    float* w3 = b2 + H;
    float* x = w3 + H;
    float* h1 = x + TS * d;
    float* h2 = h1 + TS * H;
    float* g2 = h2 + TS * H;
    float* g1 = g2 + TS * H;
    float* dy = g1 + TS * H;
    float* red = dy + TS;   /* 3 x 4 x H */
    float* lred = red + 3 * 4 * H; /* 8 */
    const int t = threadIdx.x, j = t & (H - 1), r = t >> 6, lane = t & 31, warp = t >> 5;
    for (int i = t; i < L.b3; i += NT) w1[i] = params[i]; /* w1, b1, w2, b2, w3 are contiguous */
    const float b3 = params[L.b3];
    if (BWD && step && blockIdx.x == 0 && t == 0) atomicAdd(step, 1);
    const float inv_n = 1.0f / (float)n;
    float gw1[16], gw2[16];
#pragma unroll
    for (int i = 0; i < 16; i++) gw1[i] = gw2[i] = 0.f;
    float gb1 = 0.f, gb2 = 0.f, gw3 = 0.f, gb3 = 0.f, loss = 0.f;
    __syncthreads();
    const int ntiles = (n + TS - 1) / TS;
    for (int tile = blockIdx.x; tile < ntiles; tile += gridDim.x) {
        const int s0 = tile * TS;
        const int ns = min(TS, n - s0);
        for (int i = t; i < TS * d; i += NT) {
            const int s = i / d;
            x[i] = s < ns ? X[(size_t)(s0 + s) * d + (i - s * d)] : 0.f;
        }
        __syncthreads();
        /* layer 1: thread (j, r) computes samples r, r+4, ..., r+28 of column j */
        {
            float a[8];
#pragma unroll
            for (int q = 0; q < 8; q++) a[q] = b1[j];
            for (int k = 0; k < d; k++) {
                const float w = w1[k * H + j];
#pragma unroll
                for (int q = 0; q < 8; q++) a[q] = fmaf(x[(r + 4 * q) * d + k], w, a[q]);
            }
#pragma unroll
            for (int q = 0; q < 8; q++) h1[(r + 4 * q) * H + j] = tanhf(a[q]);
        }
        __syncthreads();
        {
            float a[8];
#pragma unroll
            for (int q = 0; q < 8; q++) a[q] = b2[j];
#pragma unroll 4
            for (int k = 0; k < H; k++) {
                const float w = w2[k * H + j];
#pragma unroll
                for (int q = 0; q < 8; q++) a[q] = fmaf(h1[(r + 4 * q) * H + k], w, a[q]);
            }
#pragma unroll
            for (int q = 0; q < 8; q++) h2[(r + 4 * q) * H + j] = tanhf(a[q]);
        }
        __syncthreads();
        /* output: warp w reduces samples 4w .. 4w+3 */
#pragma unroll
        for (int i = 0; i < 4; i++) {
            const int s = warp * 4 + i;
            float v = h2[s * H + lane] * w3[lane] + h2[s * H + lane + 32] * w3[lane + 32];
#pragma unroll
            for (int o = 16; o; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
            if (lane == 0) {
                const float y = v + b3;
                if (!BWD) {
                    if (s < ns) y_out[s0 + s] = y;
                } else {
                    const float e = s < ns ? y - tgt[s0 + s] : 0.f;
                    dy[s] = 2.f * e * inv_n;
                    loss = fmaf(e * e, inv_n, loss);
                }
            }
        }
        if (!BWD) {
            __syncthreads();
            continue;
        }
        __syncthreads();
        /* dL/d(pre-activation 2), and the w3 / b2 / b3 gradients of own samples */
#pragma unroll
        for (int q = 0; q < 8; q++) {
            const int s = r + 4 * q;
            const float h = h2[s * H + j];
            const float g = dy[s] * w3[j] * (1.f - h * h);
            g2[s * H + j] = g;
            gw3 = fmaf(dy[s], h, gw3);
            gb2 += g;
        }
        if (t == 0)
            for (int s = 0; s < TS; s++) gb3 += dy[s];
        __syncthreads();
        /* W2 gradient (rows r, r+4, ..., columns j) and dL/d(pre-activation 1) */
        for (int s = 0; s < TS; s++) {
            const float gj = g2[s * H + j];
#pragma unroll
            for (int i = 0; i < 16; i++) gw2[i] = fmaf(h1[s * H + r + 4 * i], gj, gw2[i]);
        }
#pragma unroll
        for (int q = 0; q < 8; q++) {
            const int s = r + 4 * q;
            float a = 0.f;
            /* rotated column order keeps the 32 lanes on distinct banks */
#pragma unroll 8
            for (int jj = 0; jj < H; jj++) {
                const int c = (jj + j) & (H - 1);
                a = fmaf(g2[s * H + c], w2[j * H + c], a);
            }
            const float h = h1[s * H + j];
            const float g = a * (1.f - h * h);
            g1[s * H + j] = g;
            gb1 += g;
        }
        __syncthreads();
        for (int s = 0; s < TS; s++) {
            const float gj = g1[s * H + j];
#pragma unroll
            for (int i = 0; i < 16; i++) {
                const int k = r + 4 * i;
                if (k < d) gw1[i] = fmaf(x[s * d + k], gj, gw1[i]);
            }
        }
        __syncthreads();
    }
    if (!BWD) return;
    /* partial gradient row of this CTA */
    float* row = part + (size_t)blockIdx.x * L.p;
#pragma unroll
    for (int i = 0; i < 16; i++) {
        const int k = r + 4 * i;
        if (k < d) row[L.w1 + k * H + j] = gw1[i];
        row[L.w2 + k * H + j] = gw2[i];
    }
    red[(0 * 4 + r) * H + j] = gb1;
    red[(1 * 4 + r) * H + j] = gb2;
    red[(2 * 4 + r) * H + j] = gw3;
    for (int o = 16; o; o >>= 1) loss += __shfl_xor_sync(0xffffffffu, loss, o);
    if (lane == 0) lred[warp] = loss;
    __syncthreads();
    if (t < H) {
        row[L.b1 + t] = red[0 * 4 * H + t] + red[(0 * 4 + 1) * H + t] + red[(0 * 4 + 2) * H + t] + red[(0 * 4 + 3) * H + t];
        row[L.b2 + t] = red[1 * 4 * H + t] + red[(1 * 4 + 1) * H + t] + red[(1 * 4 + 2) * H + t] + red[(1 * 4 + 3) * H + t];
        row[L.w3 + t] = red[2 * 4 * H + t] + red[(2 * 4 + 1) * H + t] + red[(2 * 4 + 2) * H + t] + red[(2 * 4 + 3) * H + t];
    }
    if (t == 0) {
        row[L.b3] = gb3;
        float l = 0.f;
        for (int w = 0; w < NT / 32; w++) l += lred[w];
        lossp[blockIdx.x] = l;
    }
}

/* Sum the partial rows in CTA order; mode 0: gradient to grad, loss to
 * loss_hist[0]; mode 1: Adam step at the step count in *step, loss of the
 * pass to loss_hist[step - 1] when it fits. */
__global__ void k_cm_reduce(const float* __restrict__ part, const float* __restrict__ lossp, int nblk, int P,
                            float* __restrict__ params, float* __restrict__ m, float* __restrict__ v,
                            float* __restrict__ grad, const int* step, float* loss_hist, int hist_cap, float lr,
                            int mode) {
    const int p = blockIdx.x * blockDim.x + threadIdx.x;
    const int ts = mode ? *step : 0;
    if (p == 0) {
        float l = 0.f;
        for (int b = 0; b < nblk; b++) l += lossp[b];
        const int at = mode ? ts - 1 : 0;
        if (at >= 0 && at < hist_cap) loss_hist[at] = l;
    }
    if (p >= P) return;
    float g = 0.f;
    for (int b = 0; b < nblk; b++) g += part[(size_t)b * P + p];
    if (!mode) {
        grad[p] = g;
        return;
    }
    const float b1 = 0.9f, b2 = 0.999f, eps = 1e-8f;
    const float mt = b1 * m[p] + (1.f - b1) * g;
    const float vt = b2 * v[p] + (1.f - b2) * g * g;
    m[p] = mt;
    v[p] = vt;
    const float c1 = 1.f - powf(b1, (float)ts), c2 = 1.f - powf(b2, (float)ts);
    params[p] -= lr * (mt / c1) / (sqrtf(vt / c2) + eps);
}

uint64_t splitmix(uint64_t& s) {
    uint64_t z = (s += 0x9E3779B97F4A7C15ULL);
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ULL;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBULL;
    return z ^ (z >> 31);
}

} // namespace

struct gfs_costmodel {
    int dev = 0, d = 0, P = 0, nblk = 1;
    size_t smem = 0;
    cudaStream_t st = nullptr;
    float *params = nullptr, *m = nullptr, *v = nullptr, *grad = nullptr, *part = nullptr, *lossp = nullptr;
    float *hist = nullptr;
    int hist_cap = 0;
    int* step = nullptr;
    float *X = nullptr, *y = nullptr, *yp = nullptr;
    int n = 0, cap_n = 0, cap_pred = 0;
    cudaGraphExec_t graph = nullptr;
    float graph_lr = 0.f;
    int graph_n = -1;
};

#define CMK(x)                                                                                                         \
    do {                                                                                                               \
        if ((x) != cudaSuccess) {                                                                                      \
            cudaGetLastError();                                                                                        \
            return -GFS_EIO;                                                                                           \
        }                                                                                                              \
    } while (0)

static int cm_grid(int n) {
    const int tiles = (n + TS - 1) / TS;
    return tiles < MAX_CTAS ? (tiles > 0 ? tiles : 1) : MAX_CTAS;
}

static int cm_reset_opt(gfs_costmodel* c) {
    CMK(cudaMemsetAsync(c->m, 0, (size_t)c->P * 4, c->st));
    CMK(cudaMemsetAsync(c->v, 0, (size_t)c->P * 4, c->st));
    CMK(cudaMemsetAsync(c->step, 0, sizeof(int), c->st));
    return 0;
}

static void cm_drop_graph(gfs_costmodel* c) {
    if (c->graph) cudaGraphExecDestroy(c->graph);
    c->graph = nullptr;
    c->graph_n = -1;
}

extern "C" {

int gfs_cm_create(int n_in, int device, unsigned long long seed, gfs_costmodel** out) {
    if (!out || n_in < 1 || n_in > DMAX) return -GFS_EINVAL;
    *out = nullptr;
    gfs_costmodel* c = new gfs_costmodel();
    c->dev = device;
    c->d = n_in;
    c->P = lay(n_in).p;
    c->smem = smem_floats(n_in) * sizeof(float);
    int rc = 0;
    std::vector<float> init((size_t)c->P, 0.f);
    {
        /* Glorot-uniform weights from a seeded splitmix64 stream, zero biases */
        const Lay L = lay(n_in);
        uint64_t s = seed;
        auto uni = [&](float a) { return (float)((double)(splitmix(s) >> 11) * (1.0 / 9007199254740992.0) * 2.0 - 1.0) * a; };
        const float a1 = sqrtf(6.f / (float)(n_in + H)), a2 = sqrtf(6.f / (float)(2 * H)), a3 = sqrtf(6.f / (float)(H + 1));
        for (int i = 0; i < n_in * H; i++) init[(size_t)(L.w1 + i)] = uni(a1);
        for (int i = 0; i < H * H; i++) init[(size_t)(L.w2 + i)] = uni(a2);
        for (int i = 0; i < H; i++) init[(size_t)(L.w3 + i)] = uni(a3);
    }
    if (cudaSetDevice(device) != cudaSuccess ||
        cudaStreamCreateWithFlags(&c->st, cudaStreamNonBlocking) != cudaSuccess ||
        cudaMalloc(&c->params, (size_t)c->P * 4) != cudaSuccess || cudaMalloc(&c->m, (size_t)c->P * 4) != cudaSuccess ||
        cudaMalloc(&c->v, (size_t)c->P * 4) != cudaSuccess || cudaMalloc(&c->grad, (size_t)c->P * 4) != cudaSuccess ||
        cudaMalloc(&c->part, (size_t)MAX_CTAS * c->P * 4) != cudaSuccess ||
        cudaMalloc(&c->lossp, (size_t)MAX_CTAS * 4) != cudaSuccess || cudaMalloc(&c->step, sizeof(int)) != cudaSuccess ||
        /* the attribute is per kernel, not per model: allow the widest input */
        cudaFuncSetAttribute(k_cm_pass<true>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                             (int)(smem_floats(DMAX) * sizeof(float))) != cudaSuccess ||
        cudaFuncSetAttribute(k_cm_pass<false>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                             (int)(smem_floats(DMAX) * sizeof(float))) != cudaSuccess) {
        cudaGetLastError();
        rc = -GFS_EIO;
    }
    if (!rc) rc = gfs_cm_set_params(c, init.data());
    if (rc) {
        gfs_cm_destroy(c);
        return rc;
    }
    *out = c;
    return 0;
}

int gfs_cm_destroy(gfs_costmodel* c) {
    if (!c) return 0;
    cudaSetDevice(c->dev);
    if (c->st) cudaStreamSynchronize(c->st);
    cm_drop_graph(c);
    cudaFree(c->params);
    cudaFree(c->m);
    cudaFree(c->v);
    cudaFree(c->grad);
    cudaFree(c->part);
    cudaFree(c->lossp);
    cudaFree(c->step);
    cudaFree(c->hist);
    cudaFree(c->X);
    cudaFree(c->y);
    cudaFree(c->yp);
    if (c->st) cudaStreamDestroy(c->st);
    cudaGetLastError();
    delete c;
    return 0;
}

int gfs_cm_n_params(const gfs_costmodel* c) { return c ? c->P : -GFS_EINVAL; }

int gfs_cm_get_params(gfs_costmodel* c, float* host_out) {
    if (!c || !host_out) return -GFS_EINVAL;
    CMK(cudaSetDevice(c->dev));
    CMK(cudaMemcpyAsync(host_out, c->params, (size_t)c->P * 4, cudaMemcpyDeviceToHost, c->st));
    CMK(cudaStreamSynchronize(c->st));
    return 0;
}

int gfs_cm_set_params(gfs_costmodel* c, const float* host_in) {
    if (!c || !host_in) return -GFS_EINVAL;
    CMK(cudaSetDevice(c->dev));
    CMK(cudaMemcpyAsync(c->params, host_in, (size_t)c->P * 4, cudaMemcpyHostToDevice, c->st));
    int rc = cm_reset_opt(c);
    if (rc) return rc;
    CMK(cudaStreamSynchronize(c->st));
    return 0;
}

int gfs_cm_set_data(gfs_costmodel* c, const float* X, const float* y, int n) {
    if (!c || !X || !y || n < 1) return -GFS_EINVAL;
    CMK(cudaSetDevice(c->dev));
    if (n > c->cap_n) {
        CMK(cudaStreamSynchronize(c->st));
        cudaFree(c->X);
        cudaFree(c->y);
        c->X = c->y = nullptr;
        c->cap_n = 0;
        CMK(cudaMalloc(&c->X, (size_t)n * c->d * 4));
        CMK(cudaMalloc(&c->y, (size_t)n * 4));
        c->cap_n = n;
        cm_drop_graph(c);
    }
    CMK(cudaMemcpyAsync(c->X, X, (size_t)n * c->d * 4, cudaMemcpyHostToDevice, c->st));
    CMK(cudaMemcpyAsync(c->y, y, (size_t)n * 4, cudaMemcpyHostToDevice, c->st));
    CMK(cudaStreamSynchronize(c->st));
    if (n != c->n) cm_drop_graph(c);
    c->n = n;
    c->nblk = cm_grid(n);
    return 0;
}

static int cm_hist(gfs_costmodel* c, int need) {
    if (need <= c->hist_cap) return 0;
    CMK(cudaStreamSynchronize(c->st));
    cudaFree(c->hist);
    c->hist = nullptr;
    c->hist_cap = 0;
    CMK(cudaMalloc(&c->hist, (size_t)need * 4));
    c->hist_cap = need;
    cm_drop_graph(c);
    return 0;
}

int gfs_cm_grad(gfs_costmodel* c, float* host_grad, float* host_loss) {
    if (!c || !host_grad || c->n < 1) return -GFS_EINVAL;
    CMK(cudaSetDevice(c->dev));
    int rc = cm_hist(c, 1);
    if (rc) return rc;
    k_cm_pass<true><<<c->nblk, NT, c->smem, c->st>>>(c->params, c->X, c->y, c->n, c->d, c->part, c->lossp, nullptr,
                                                      nullptr);
    k_cm_reduce<<<(c->P + 255) / 256, 256, 0, c->st>>>(c->part, c->lossp, c->nblk, c->P, c->params, c->m, c->v,
                                                       c->grad, c->step, c->hist, c->hist_cap, 0.f, 0);
    CMK(cudaGetLastError());
    CMK(cudaMemcpyAsync(host_grad, c->grad, (size_t)c->P * 4, cudaMemcpyDeviceToHost, c->st));
    float l = 0.f;
    CMK(cudaMemcpyAsync(&l, c->hist, 4, cudaMemcpyDeviceToHost, c->st));
    CMK(cudaStreamSynchronize(c->st));
    if (host_loss) *host_loss = l;
    return 0;
}

static void cm_step(gfs_costmodel* c, float lr) {
    k_cm_pass<true><<<c->nblk, NT, c->smem, c->st>>>(c->params, c->X, c->y, c->n, c->d, c->part, c->lossp, nullptr,
                                                      c->step);
    k_cm_reduce<<<(c->P + 255) / 256, 256, 0, c->st>>>(c->part, c->lossp, c->nblk, c->P, c->params, c->m, c->v,
                                                       c->grad, c->step, c->hist, c->hist_cap, lr, 1);
}

int gfs_cm_train(gfs_costmodel* c, int steps, float lr, float* host_losses) {
    if (!c || steps < 0 || c->n < 1 || !(lr > 0.f)) return -GFS_EINVAL;
    if (steps == 0) return 0;
    CMK(cudaSetDevice(c->dev));
    int rc = cm_reset_opt(c);
    if (!rc) rc = cm_hist(c, steps);
    if (rc) return rc;
    /* launch-bound loop: GRAPH_STEPS steps per captured graph */
    if (steps >= GRAPH_STEPS && (!c->graph || c->graph_lr != lr || c->graph_n != c->n)) {
        cm_drop_graph(c);
        cudaGraph_t gr = nullptr;
        CMK(cudaStreamBeginCapture(c->st, cudaStreamCaptureModeThreadLocal));
        for (int i = 0; i < GRAPH_STEPS; i++) cm_step(c, lr);
        const cudaError_t e = cudaStreamEndCapture(c->st, &gr);
        if (e != cudaSuccess || cudaGraphInstantiate(&c->graph, gr, 0) != cudaSuccess) {
            if (gr) cudaGraphDestroy(gr);
            c->graph = nullptr;
            cudaGetLastError();
            return -GFS_EIO;
        }
        cudaGraphDestroy(gr);
        c->graph_lr = lr;
        c->graph_n = c->n;
    }
    int done = 0;
    for (; c->graph && done + GRAPH_STEPS <= steps; done += GRAPH_STEPS) CMK(cudaGraphLaunch(c->graph, c->st));
    for (; done < steps; done++) cm_step(c, lr);
    CMK(cudaGetLastError());
    if (host_losses) CMK(cudaMemcpyAsync(host_losses, c->hist, (size_t)steps * 4, cudaMemcpyDeviceToHost, c->st));
    CMK(cudaStreamSynchronize(c->st));
    return 0;
}

int gfs_cm_predict(gfs_costmodel* c, const float* X, int n, float* host_y) {
    if (!c || !X || !host_y || n < 1) return -GFS_EINVAL;
    CMK(cudaSetDevice(c->dev));
    if (n > c->cap_pred) {
        CMK(cudaStreamSynchronize(c->st));
        cudaFree(c->yp);
        c->yp = nullptr;
        c->cap_pred = 0;
        CMK(cudaMalloc(&c->yp, (size_t)n * (c->d + 1) * 4));
        c->cap_pred = n;
    }
    float* xp = c->yp + n;
    CMK(cudaMemcpyAsync(xp, X, (size_t)n * c->d * 4, cudaMemcpyHostToDevice, c->st));
    k_cm_pass<false><<<cm_grid(n), NT, c->smem, c->st>>>(c->params, xp, nullptr, n, c->d, nullptr, nullptr, c->yp,
                                                          nullptr);
    CMK(cudaGetLastError());
    CMK(cudaMemcpyAsync(host_y, c->yp, (size_t)n * 4, cudaMemcpyDeviceToHost, c->st));
    CMK(cudaStreamSynchronize(c->st));
    return 0;
}

} /* extern "C" */
