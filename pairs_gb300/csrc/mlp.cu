// Learned rebuild schedule: per-cell features, a 3-64-64-1 FP32 MLP, its training.
//
// The reference rebuilds its Verlet lists on a fixed period
// (sim/simulation.py:232-233, predicate sim/timestep.py:47).  Here a small network
// predicts, per cell, log(steps until a particle of the cell has moved more than
// skin/2 since the last build) from
//   f0 = max |v| * dt / (skin/2)        (fastest particle, in half-skins per step)
//   f1 = mean |F| / m * dt^2 / (skin/2)  (mean acceleration, same units)
//   f2 = steps since the last build / 20
// and the system prediction is a soft minimum over non-empty cells,
//   P = m - T log sum_c exp(-(o_c - m) / T),  m = min_c o_c.
// The exact FP64 displacement guard (integrate.cu) stays in charge: the prediction
// only decides when to rebuild before the guard trips.
//
// Parameters (FP32, contiguous): W1[64][3] b1[64] W2[64][64] b2[64] W3[64] b3.
// Loss of one sample with target R (steps remaining, observed):
//   e = P - log R;  L = e^2 (trip observed) or min(e, 0)^2 (censored: R is a lower
//   bound).  dL/do_c = dL/dP * softmax(-o/T)_c.
#include "common.cuh"

namespace pg {

constexpr int kH = 64;
constexpr int kIn = 3;
constexpr int kOffW1 = 0, kOffB1 = kOffW1 + kH * kIn, kOffW2 = kOffB1 + kH, kOffB2 = kOffW2 + kH * kH;
constexpr int kOffW3 = kOffB2 + kH, kOffB3 = kOffW3 + kH, kParams = kOffB3 + 1;
constexpr int kFeat = 4;   // f0, f1, f2, valid

// ---------------------------------------------------------------- features

__global__ void k_cell_features(pg_particles p, pg_cells cells, int precision, float since, float dt,
                                float inv_half_skin, float *feat) {
    const int warp = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const int lane = threadIdx.x & 31;
    if(warp >= cells.ncells) { return; }
    const int b = cells.cell_start[warp], cnt = cells.cell_count[warp];
    float vmax = 0.0f, fsum = 0.0f;
    for(int k = lane; k < cnt; k += 32) {
        const int i = b + k;
        const D4 v = ld_d4(p.vel, i);
        const float vv = (float) (v.x * v.x + v.y * v.y + v.z * v.z);
        vmax = fmaxf(vmax, vv);
        float fx, fy, fz;
        if(precision == PG_MIXED) {
            const float4 f = ld_f4(p.force32, i);
            fx = f.x; fy = f.y; fz = f.z;
        } else {
            const D4 f = ld_d4(p.force, i);
            fx = (float) f.x; fy = (float) f.y; fz = (float) f.z;
        }
        fsum += sqrtf(fx * fx + fy * fy + fz * fz) / (float) p.mass[i];
    }
    for(int o = 16; o > 0; o >>= 1) {
        vmax = fmaxf(vmax, __shfl_xor_sync(0xffffffffu, vmax, o));
        fsum += __shfl_xor_sync(0xffffffffu, fsum, o);
    }
    if(lane == 0) {
        float *f = feat + (size_t) warp * kFeat;
        f[0] = sqrtf(vmax) * dt * inv_half_skin;
        f[1] = cnt > 0 ? fsum / cnt * dt * dt * inv_half_skin : 0.0f;
        f[2] = since * (1.0f / 20.0f);
        f[3] = cnt > 0 ? 1.0f : 0.0f;
    }
}

// ---------------------------------------------------------------- forward

__device__ __forceinline__ void load_params(const float *params, float *s) {
    for(int k = threadIdx.x; k < kParams; k += blockDim.x) { s[k] = params[k]; }
    __syncthreads();
}

__device__ __forceinline__ float mlp_eval(const float *s, const float *x, float *h1) {
    for(int u = 0; u < kH; u++) {
        float z = s[kOffB1 + u];
        for(int k = 0; k < kIn; k++) { z = fmaf(s[kOffW1 + u * kIn + k], x[k], z); }
        h1[u] = tanhf(z);
    }
    float o = s[kOffB3];
    for(int u = 0; u < kH; u++) {
        float z = s[kOffB2 + u];
        const float *w = s + kOffW2 + u * kH;
        #pragma unroll 16
        for(int k = 0; k < kH; k++) { z = fmaf(w[k], h1[k], z); }
        o = fmaf(s[kOffW3 + u], tanhf(z), o);
    }
    return o;
}

__global__ void __launch_bounds__(128) k_mlp_forward(const float *params, const float *feat, int ncells,
                                                     float *out) {
    __shared__ float s[kParams];
    load_params(params, s);
    const int c = blockIdx.x * blockDim.x + threadIdx.x;
    if(c >= ncells) { return; }
    const float *f = feat + (size_t) c * kFeat;
    float h1[kH];
    const float x[kIn] = {f[0], f[1], f[2]};
    out[c] = f[3] > 0.0f ? mlp_eval(s, x, h1) : INFINITY;
}

// ---------------------------------------------------------------- soft minimum

__device__ __forceinline__ int float_to_ordered(float f) {
    const int i = __float_as_int(f);
    return i >= 0 ? i : i ^ 0x7fffffff;
}

__device__ __forceinline__ float ordered_to_float(int i) {
    return __int_as_float(i >= 0 ? i : i ^ 0x7fffffff);
}

// result: [0] soft-min P, [1] min (ordered int bits), [2] sum of exp, [3] loss accumulator
__global__ void k_softmin_min(const float *out, int n, int *min_bits) {
    int m = float_to_ordered(INFINITY);
    for(int c = blockIdx.x * blockDim.x + threadIdx.x; c < n; c += gridDim.x * blockDim.x) {
        m = min(m, float_to_ordered(out[c]));
    }
    for(int o = 16; o > 0; o >>= 1) { m = min(m, __shfl_xor_sync(0xffffffffu, m, o)); }
    if((threadIdx.x & 31) == 0) { atomicMin(min_bits, m); }
}

__global__ void k_softmin_sum(const float *out, int n, float inv_t, float *result) {
    const float m = ordered_to_float(*reinterpret_cast<const int *>(result + 1));
    float s = 0.0f;
    for(int c = blockIdx.x * blockDim.x + threadIdx.x; c < n; c += gridDim.x * blockDim.x) {
        const float o = out[c];
        if(o < INFINITY) { s += __expf(-(o - m) * inv_t); }
    }
    for(int o = 16; o > 0; o >>= 1) { s += __shfl_xor_sync(0xffffffffu, s, o); }
    if((threadIdx.x & 31) == 0) { atomicAdd(result + 2, s); }
}

__global__ void k_softmin_init(float *result) {
    reinterpret_cast<int *>(result)[1] = 0x7f800000;      // ordered bits of +inf
    result[2] = 0.0f;
}

__global__ void k_softmin_finish(float temperature, float *result) {
    const float m = ordered_to_float(*reinterpret_cast<const int *>(result + 1));
    result[0] = m - temperature * logf(fmaxf(result[2], 1e-30f));
}

// ---------------------------------------------------------------- backward

// grads (kParams) accumulate over cells and samples; loss accumulates in *loss.
// One block walks the sample's cells in chunks of blockDim.x: every thread computes
// its cell's activations and local gradients (dL/dz2, dL/dz1) into shared memory,
// then each thread owns a fixed slice of the parameters and sums that slice over the
// chunk (no atomics on shared data); the block adds each parameter's total to the
// global gradient once.
constexpr int kBwdThreads = 128;

__global__ void __launch_bounds__(kBwdThreads) k_mlp_backward(const float *params, const float *feat,
                                                             const float *out, int ncells, const float *result,
                                                             float target_log, int censored, float inv_t,
                                                             float *grads, float *loss) {
    __shared__ float s[kParams];
    extern __shared__ float dyn[];
    float *H1 = dyn;                              // [kBwdThreads][kH]
    float *DZ2 = H1 + kBwdThreads * kH;           // [kBwdThreads][kH]
    float *DZ1 = DZ2 + kBwdThreads * kH;          // [kBwdThreads][kH]
    float *X = DZ1 + kBwdThreads * kH;            // [kBwdThreads][4]: x0, x1, x2, go
    float *H2 = X + kBwdThreads * 4;              // [kBwdThreads][kH]
    load_params(params, s);
    const float P = result[0];
    const float m = ordered_to_float(*reinterpret_cast<const int *>(result + 1));
    const float Z = fmaxf(result[2], 1e-30f);
    float e = P - target_log;
    if(censored) { e = fminf(e, 0.0f); }
    const float dP = 2.0f * e;
    if(threadIdx.x == 0) { atomicAdd(loss, e * e); }
    // parameter slice owned by this thread: W2 entries t, t+T, ...; then the small ones
    float acc[kH * kH / kBwdThreads];
    float acc_small[(kParams - kH * kH + kBwdThreads - 1) / kBwdThreads];
    for(int q = 0; q < kH * kH / kBwdThreads; q++) { acc[q] = 0.0f; }
    for(int q = 0; q < (int) (sizeof(acc_small) / sizeof(float)); q++) { acc_small[q] = 0.0f; }
    const int t = threadIdx.x;
    for(int c0 = 0; c0 < ncells; c0 += kBwdThreads) {
        const int c = c0 + t;
        float w = 0.0f;
        if(c < ncells && out[c] < INFINITY) { w = __expf(-(out[c] - m) * inv_t) / Z; }
        const float go = dP * w;
        const bool active = go != 0.0f;
        if(!__syncthreads_or(active)) { continue; }
        float *h1 = H1 + t * kH, *dz2 = DZ2 + t * kH, *dz1 = DZ1 + t * kH, *h2 = H2 + t * kH;
        float x[kIn] = {0.0f, 0.0f, 0.0f};
        if(active) {
            const float *f = feat + (size_t) c * kFeat;
            x[0] = f[0]; x[1] = f[1]; x[2] = f[2];
            for(int u = 0; u < kH; u++) {
                float z = s[kOffB1 + u];
                for(int k = 0; k < kIn; k++) { z = fmaf(s[kOffW1 + u * kIn + k], x[k], z); }
                h1[u] = tanhf(z);
                dz1[u] = 0.0f;
            }
            for(int u = 0; u < kH; u++) {
                float z = s[kOffB2 + u];
                const float *wr = s + kOffW2 + u * kH;
                for(int k = 0; k < kH; k++) { z = fmaf(wr[k], h1[k], z); }
                const float hz = tanhf(z);
                h2[u] = hz;
                const float d2 = go * s[kOffW3 + u] * (1.0f - hz * hz);
                dz2[u] = d2;
                for(int k = 0; k < kH; k++) { dz1[k] = fmaf(d2, wr[k], dz1[k]); }
            }
            for(int u = 0; u < kH; u++) { dz1[u] *= (1.0f - h1[u] * h1[u]); }
        } else {
            for(int u = 0; u < kH; u++) { h1[u] = 0.0f; dz2[u] = 0.0f; dz1[u] = 0.0f; h2[u] = 0.0f; }
        }
        X[t * 4 + 0] = x[0]; X[t * 4 + 1] = x[1]; X[t * 4 + 2] = x[2]; X[t * 4 + 3] = go;
        __syncthreads();
        // W2[u][k] += sum_c dz2[c][u] h1[c][k]
        for(int q = 0; q < kH * kH / kBwdThreads; q++) {
            const int e2 = t + q * kBwdThreads, u = e2 / kH, k = e2 % kH;
            float a = 0.0f;
            for(int cc = 0; cc < kBwdThreads; cc++) { a = fmaf(DZ2[cc * kH + u], H1[cc * kH + k], a); }
            acc[q] += a;
        }
        // the rest: W1[u][k] (dz1 x), b1 (dz1), b2 (dz2), W3 (go h2), b3 (go)
        for(int q = 0; q < (int) (sizeof(acc_small) / sizeof(float)); q++) {
            const int r = t + q * kBwdThreads;
            float a = 0.0f;
            if(r < kH * kIn) {
                const int u = r / kIn, k = r % kIn;
                for(int cc = 0; cc < kBwdThreads; cc++) { a = fmaf(DZ1[cc * kH + u], X[cc * 4 + k], a); }
            } else if(r < kH * kIn + kH) {
                const int u = r - kH * kIn;
                for(int cc = 0; cc < kBwdThreads; cc++) { a += DZ1[cc * kH + u]; }
            } else if(r < kH * kIn + 2 * kH) {
                const int u = r - kH * kIn - kH;
                for(int cc = 0; cc < kBwdThreads; cc++) { a += DZ2[cc * kH + u]; }
            } else if(r < kH * kIn + 3 * kH) {
                const int u = r - kH * kIn - 2 * kH;
                for(int cc = 0; cc < kBwdThreads; cc++) { a = fmaf(X[cc * 4 + 3], H2[cc * kH + u], a); }
            } else if(r == kH * kIn + 3 * kH) {
                for(int cc = 0; cc < kBwdThreads; cc++) { a += X[cc * 4 + 3]; }
            }
            acc_small[q] += a;
        }
        __syncthreads();
    }
    for(int q = 0; q < kH * kH / kBwdThreads; q++) {
        const int e2 = t + q * kBwdThreads;
        if(acc[q] != 0.0f) { atomicAdd(&grads[kOffW2 + e2], acc[q]); }
    }
    for(int q = 0; q < (int) (sizeof(acc_small) / sizeof(float)); q++) {
        const int r = t + q * kBwdThreads;
        if(acc_small[q] == 0.0f) { continue; }
        int dst;
        if(r < kH * kIn) { dst = kOffW1 + r; }
        else if(r < kH * kIn + kH) { dst = kOffB1 + (r - kH * kIn); }
        else if(r < kH * kIn + 2 * kH) { dst = kOffB2 + (r - kH * kIn - kH); }
        else if(r < kH * kIn + 3 * kH) { dst = kOffW3 + (r - kH * kIn - 2 * kH); }
        else if(r == kH * kIn + 3 * kH) { dst = kOffB3; }
        else { continue; }
        atomicAdd(&grads[dst], acc_small[q]);
    }
}

// ---------------------------------------------------------------- Adam

__global__ void k_adam(float *params, float *grads, float *m1, float *m2, int n, float lr, float b1, float b2,
                       float eps, float c1, float c2, float scale) {
    const int k = blockIdx.x * blockDim.x + threadIdx.x;
    if(k >= n) { return; }
    const float gk = grads[k] * scale;
    const float a = b1 * m1[k] + (1.0f - b1) * gk;
    const float b = b2 * m2[k] + (1.0f - b2) * gk * gk;
    m1[k] = a; m2[k] = b;
    params[k] -= lr * (a / c1) / (sqrtf(b / c2) + eps);
    grads[k] = 0.0f;
}

// ---------------------------------------------------------------- host side

int cell_features(const pg_particles *p, const pg_cells *cells, int precision, int32_t since, double dt,
                  double half_skin, float *feat, cudaStream_t st) {
    if(!p || !cells || !feat || !p->vel || !p->mass) { return PG_ERR_ARGUMENT; }
    if(precision == PG_MIXED ? !p->force32 : !p->force) { return PG_ERR_ARGUMENT; }
    const int threads = 256;
    const int blocks = (int) (((int64_t) cells->ncells * 32 + threads - 1) / threads);
    k_cell_features<<<blocks, threads, 0, st>>>(*p, *cells, precision, (float) since, (float) dt,
                                                 (float) (1.0 / half_skin), feat); note_launch();
    return launch_status();
}

int mlp_forward(const float *params, const float *feat, int32_t ncells, float *out, cudaStream_t st) {
    if(!params || !feat || !out || ncells <= 0) { return PG_ERR_ARGUMENT; }
    k_mlp_forward<<<blocks_for(ncells, 128), 128, 0, st>>>(params, feat, ncells, out); note_launch();
    return launch_status();
}

int mlp_softmin(const float *out, int32_t ncells, float temperature, float *result, cudaStream_t st) {
    if(!out || !result || ncells <= 0 || !(temperature > 0.0f)) { return PG_ERR_ARGUMENT; }
    k_softmin_init<<<1, 1, 0, st>>>(result); note_launch();
    const int blocks = min(blocks_for(ncells), 4 * kSMs);
    k_softmin_min<<<blocks, kBlock, 0, st>>>(out, ncells, reinterpret_cast<int *>(result + 1)); note_launch();
    k_softmin_sum<<<blocks, kBlock, 0, st>>>(out, ncells, 1.0f / temperature, result); note_launch();
    k_softmin_finish<<<1, 1, 0, st>>>(temperature, result); note_launch();
    return launch_status();
}

int mlp_backward(const float *params, const float *feat, const float *out, int32_t ncells, const float *result,
                 float target_log, int censored, float temperature, float *grads, float *loss, cudaStream_t st) {
    if(!params || !feat || !out || !result || !grads || !loss || ncells <= 0) { return PG_ERR_ARGUMENT; }
    const size_t smem = (size_t) kBwdThreads * (4 * kH + 4) * sizeof(float);
    if(cudaFuncSetAttribute(k_mlp_backward, cudaFuncAttributeMaxDynamicSharedMemorySize, (int) smem) != cudaSuccess) {
        return PG_ERR_CUDA;
    }
    k_mlp_backward<<<1, kBwdThreads, smem, st>>>(params, feat, out, ncells, result, target_log, censored,
                                                   1.0f / temperature, grads, loss);
    note_launch();
    return launch_status();
}

int mlp_adam(float *params, float *grads, float *m1, float *m2, float lr, float b1, float b2, float eps,
             int32_t t, float scale, cudaStream_t st) {
    if(!params || !grads || !m1 || !m2 || t < 1) { return PG_ERR_ARGUMENT; }
    const float c1 = 1.0f - powf(b1, (float) t), c2 = 1.0f - powf(b2, (float) t);
    k_adam<<<blocks_for(kParams), kBlock, 0, st>>>(params, grads, m1, m2, kParams, lr, b1, b2, eps, c1, c2, scale);
    note_launch();
    return launch_status();
}

int mlp_param_count() { return kParams; }

}  // namespace pg
