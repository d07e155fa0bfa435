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

// One thread per particle (particles are stored in cell order, so a warp spans a few
// cells): each lane adds its particle's |F|/m to its cell with an atomic, and the
// lanes of a cell take the largest |v|^2 together (redux over the lanes that share the
// cell) before one of them publishes it.  The accumulators live in the feature rows
// themselves (zeroed first); k_cell_finish turns them into the features.  (A kernel
// with 16 lanes per cell of ~10 particles took 39 us at 1M atoms in 110k cells.)
// With perm (a binning's permutation, perm[k] = index before the binning of particle k),
// the state was just binned: every array is in the new order except the forces, which
// the binning leaves in the old one.
__global__ void __launch_bounds__(256) k_cell_accum(pg_particles p, pg_cells cells, int precision,
                                                    const int32_t *perm, float *feat) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    const int c = i < p.n ? cells.particle_cell[i] : -1;
    const bool live = c >= 0 && c < cells.ncells;
    float vv = 0.0f, fm = 0.0f;
    if(live) {
        const D4 v = ld_d4(p.vel, i);
        vv = (float) (v.x * v.x + v.y * v.y + v.z * v.z);
        float fx, fy, fz;
        const int fi = perm != nullptr ? perm[i] : i;
        if(precision == PG_MIXED) {
            const float4 f = ld_f4(p.force32, fi);
            fx = f.x; fy = f.y; fz = f.z;
        } else {
            const D4 f = ld_d4(p.force, fi);
            fx = (float) f.x; fy = (float) f.y; fz = (float) f.z;
        }
        fm = sqrtf(fx * fx + fy * fy + fz * fz) / (float) p.mass[i];
    }
    const unsigned group = __match_any_sync(0xffffffffu, c);
    // |v|^2 >= 0: its bit pattern orders like the value
    const int vmax = __reduce_max_sync(group, __float_as_int(vv));
    if(live) {
        float *f = feat + (size_t) c * kFeat;
        atomicAdd(f + 1, fm);
        if((threadIdx.x & 31) == (unsigned) (__ffs(group) - 1)) { atomicMax(reinterpret_cast<int *>(f), vmax); }
    }
}

__global__ void __launch_bounds__(256) k_cell_finish(pg_cells cells, float since, float dt, float inv_half_skin,
                                                     float *feat) {
    const int c = blockIdx.x * blockDim.x + threadIdx.x;
    if(c >= cells.ncells) { return; }
    float *f = feat + (size_t) c * kFeat;
    const int cnt = cells.cell_count[c];
    const float vmax = __int_as_float(*reinterpret_cast<const int *>(f));
    f[0] = sqrtf(vmax) * dt * inv_half_skin;
    f[1] = cnt > 0 ? f[1] / cnt * dt * dt * inv_half_skin : 0.0f;
    f[2] = since * (1.0f / 20.0f);
    f[3] = cnt > 0 ? 1.0f : 0.0f;
}

// ---------------------------------------------------------------- forward

__device__ __forceinline__ void load_params(const float *params, float *s) {
    for(int k = threadIdx.x; k < kParams; k += blockDim.x) { s[k] = params[k]; }
    __syncthreads();
}

// One warp evaluates one cell: lane l owns hidden units l and l + 32 of both layers;
// the first layer's activations reach every lane through shuffles.
struct WarpAct {
    float h1a, h1b;      // tanh of layer 1, units l and l+32
    float h2a, h2b;      // tanh of layer 2
};

__device__ __forceinline__ float warp_mlp(const float *s, const float x[kIn], WarpAct &act) {
    const int l = threadIdx.x & 31;
    float za = s[kOffB1 + l], zb = s[kOffB1 + l + 32];
    for(int k = 0; k < kIn; k++) {
        za = fmaf(s[kOffW1 + l * kIn + k], x[k], za);
        zb = fmaf(s[kOffW1 + (l + 32) * kIn + k], x[k], zb);
    }
    act.h1a = tanhf(za);
    act.h1b = tanhf(zb);
    float ya = s[kOffB2 + l], yb = s[kOffB2 + l + 32];
    const float *wa = s + kOffW2 + l * kH, *wb = s + kOffW2 + (l + 32) * kH;
    #pragma unroll 8
    for(int j = 0; j < 32; j++) {
        const float p = __shfl_sync(0xffffffffu, act.h1a, j), q = __shfl_sync(0xffffffffu, act.h1b, j);
        ya = fmaf(wa[j], p, ya); ya = fmaf(wa[j + 32], q, ya);
        yb = fmaf(wb[j], p, yb); yb = fmaf(wb[j + 32], q, yb);
    }
    act.h2a = tanhf(ya);
    act.h2b = tanhf(yb);
    float o = s[kOffW3 + l] * act.h2a + s[kOffW3 + l + 32] * act.h2b;
    for(int off = 16; off > 0; off >>= 1) { o += __shfl_xor_sync(0xffffffffu, o, off); }
    return o + s[kOffB3];
}

constexpr int kFwdThreads = 256;

__global__ void __launch_bounds__(kFwdThreads) k_mlp_forward(const float *params, const float *feat, int ncells,
                                                             float *out) {
    __shared__ float s[kParams];
    load_params(params, s);
    const int c = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    if(c >= ncells) { return; }
    const float *f = feat + (size_t) c * kFeat;
    const float x[kIn] = {f[0], f[1], f[2]};
    WarpAct act;
    const float o = warp_mlp(s, x, act);
    if((threadIdx.x & 31) == 0) { out[c] = f[3] > 0.0f ? o : INFINITY; }
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

// One block for a few thousand cells: min, partition sum and soft-min in one launch.
constexpr int kSoftminBlock = 1024;
constexpr int kSoftminOneBlockMax = 16384;

__global__ void __launch_bounds__(kSoftminBlock) k_softmin_block(const float *out, int n, float temperature,
                                                                float *result) {
    __shared__ int smin[kSoftminBlock / 32];
    __shared__ float ssum[kSoftminBlock / 32];
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nw = blockDim.x >> 5;
    int m = float_to_ordered(INFINITY);
    for(int c = threadIdx.x; c < n; c += blockDim.x) { m = min(m, float_to_ordered(out[c])); }
    for(int o = 16; o > 0; o >>= 1) { m = min(m, __shfl_xor_sync(0xffffffffu, m, o)); }
    if(lane == 0) { smin[warp] = m; }
    __syncthreads();
    m = smin[0];
    for(int w = 1; w < nw; w++) { m = min(m, smin[w]); }
    const float mf = ordered_to_float(m), inv_t = 1.0f / temperature;
    float s = 0.0f;
    for(int c = threadIdx.x; c < n; c += blockDim.x) {
        const float o = out[c];
        if(o < INFINITY) { s += __expf(-(o - mf) * inv_t); }
    }
    for(int o = 16; o > 0; o >>= 1) { s += __shfl_xor_sync(0xffffffffu, s, o); }
    if(lane == 0) { ssum[warp] = s; }
    __syncthreads();
    if(threadIdx.x == 0) {
        float z = 0.0f;
        for(int w = 0; w < nw; w++) { z += ssum[w]; }
        reinterpret_cast<int *>(result)[1] = m;
        result[2] = z;
        result[0] = mf - temperature * logf(fmaxf(z, 1e-30f));
    }
}

// The sample's cells: ncells features split into k contiguous groups (slabs of the
// cell grid); each group contributes its cell with the largest feature 0 (the fastest
// particle, relative to skin/2), the first one on ties.  The fastest cell of the
// system is always among them.
constexpr int kSelectThreads = 128;

__global__ void __launch_bounds__(kSelectThreads) k_cell_select(const float *feat, int ncells, int k, float *out) {
    __shared__ float sv[kSelectThreads / 32];
    __shared__ int si[kSelectThreads / 32];
    const int g = blockIdx.x;
    const int b = (int) ((int64_t) g * ncells / k), e = (int) ((int64_t) (g + 1) * ncells / k);
    float v = -INFINITY;
    int idx = b;
    for(int c = b + threadIdx.x; c < e; c += blockDim.x) {
        const float f = feat[(size_t) c * 4];
        if(f > v) { v = f; idx = c; }
    }
    for(int o = 16; o > 0; o >>= 1) {
        const float ov = __shfl_xor_sync(0xffffffffu, v, o);
        const int oi = __shfl_xor_sync(0xffffffffu, idx, o);
        if(ov > v || (ov == v && oi < idx)) { v = ov; idx = oi; }
    }
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    if(lane == 0) { sv[warp] = v; si[warp] = idx; }
    __syncthreads();
    if(threadIdx.x == 0) {
        for(int w = 1; w < (int) (blockDim.x >> 5); w++) {
            if(sv[w] > v || (sv[w] == v && si[w] < idx)) { v = sv[w]; idx = si[w]; }
        }
        si[0] = idx;
    }
    __syncthreads();
    if(threadIdx.x < 4) { out[(size_t) g * 4 + threadIdx.x] = e > b ? feat[(size_t) si[0] * 4 + threadIdx.x] : 0.0f; }
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

// Gradient of one sample's loss.  A block takes kBwdCells cells: each warp runs the
// forward and backward pass of its cells (lane l owns hidden units l and l + 32),
// writing the per-cell vectors dz2 (layer-2 pre-activation gradient), h1, dz1 and
// the cell's output gradient to shared memory; the block then forms its partial
// weight gradients (W2 as sum_c dz2 h1^T, thread-owned entries, no shared atomics)
// and adds them to the global gradient once.
constexpr int kBwdThreads = 256;
constexpr int kBwdCells = 16;
constexpr int kBwdSlice = (kParams + kBwdThreads - 1) / kBwdThreads;

__global__ void __launch_bounds__(kBwdThreads) k_mlp_backward(const float *params, const float *feat,
                                                             const float *out, int ncells, const float *result,
                                                             float target_log, int censored, float inv_t,
                                                             float *grads, float *loss) {
    __shared__ float s[kParams];
    __shared__ float H1[kBwdCells][kH], DZ2[kBwdCells][kH], DZ1[kBwdCells][kH], H2[kBwdCells][kH];
    __shared__ float X[kBwdCells][4];
    load_params(params, s);
    const float P = result[0];
    const float m = ordered_to_float(*reinterpret_cast<const int *>(result + 1));
    const float Z = fmaxf(result[2], 1e-30f);
    float e = P - target_log;
    if(censored) { e = fminf(e, 0.0f); }
    const float dP = 2.0f * e;
    if(blockIdx.x == 0 && threadIdx.x == 0) { atomicAdd(loss, e * e); }
    const int warp = threadIdx.x >> 5, l = threadIdx.x & 31;
    const int c0 = blockIdx.x * kBwdCells;
    for(int cc = warp; cc < kBwdCells; cc += kBwdThreads / 32) {
        const int c = c0 + cc;
        float go = 0.0f;
        if(c < ncells && out[c] < INFINITY) { go = dP * __expf(-(out[c] - m) * inv_t) / Z; }
        float x[kIn] = {0.0f, 0.0f, 0.0f};
        if(go != 0.0f) {
            const float *f = feat + (size_t) c * kFeat;
            x[0] = f[0]; x[1] = f[1]; x[2] = f[2];
            WarpAct act;
            warp_mlp(s, x, act);
            const float da = go * s[kOffW3 + l] * (1.0f - act.h2a * act.h2a);
            const float db = go * s[kOffW3 + l + 32] * (1.0f - act.h2b * act.h2b);
            // dz1[k] = (sum_u d2[u] W2[u][k]) (1 - h1[k]^2), k = l and l + 32
            float ga = 0.0f, gb = 0.0f;
            #pragma unroll 8
            for(int j = 0; j < 32; j++) {
                const float p = __shfl_sync(0xffffffffu, da, j), q = __shfl_sync(0xffffffffu, db, j);
                ga = fmaf(p, s[kOffW2 + j * kH + l], ga); ga = fmaf(q, s[kOffW2 + (j + 32) * kH + l], ga);
                gb = fmaf(p, s[kOffW2 + j * kH + l + 32], gb); gb = fmaf(q, s[kOffW2 + (j + 32) * kH + l + 32], gb);
            }
            H1[cc][l] = act.h1a; H1[cc][l + 32] = act.h1b;
            H2[cc][l] = act.h2a; H2[cc][l + 32] = act.h2b;
            DZ2[cc][l] = da; DZ2[cc][l + 32] = db;
            DZ1[cc][l] = ga * (1.0f - act.h1a * act.h1a);
            DZ1[cc][l + 32] = gb * (1.0f - act.h1b * act.h1b);
        } else {
            H1[cc][l] = H1[cc][l + 32] = 0.0f; H2[cc][l] = H2[cc][l + 32] = 0.0f;
            DZ2[cc][l] = DZ2[cc][l + 32] = 0.0f; DZ1[cc][l] = DZ1[cc][l + 32] = 0.0f;
        }
        if(l < 4) { X[cc][l] = l < kIn ? x[l] : go; }
    }
    __syncthreads();
    // partial gradients of this block's cells; thread t owns parameters t, t+T, ...
    for(int q = 0; q < kBwdSlice; q++) {
        const int r = threadIdx.x + q * kBwdThreads;
        if(r >= kParams) { break; }
        float a = 0.0f;
        if(r >= kOffW2 && r < kOffB2) {
            const int u = (r - kOffW2) / kH, k = (r - kOffW2) % kH;
            for(int cc = 0; cc < kBwdCells; cc++) { a = fmaf(DZ2[cc][u], H1[cc][k], a); }
        } else if(r < kOffB1) {
            const int u = r / kIn, k = r % kIn;
            for(int cc = 0; cc < kBwdCells; cc++) { a = fmaf(DZ1[cc][u], X[cc][k], a); }
        } else if(r < kOffW2) {
            const int u = r - kOffB1;
            for(int cc = 0; cc < kBwdCells; cc++) { a += DZ1[cc][u]; }
        } else if(r < kOffW3) {
            const int u = r - kOffB2;
            for(int cc = 0; cc < kBwdCells; cc++) { a += DZ2[cc][u]; }
        } else if(r < kOffB3) {
            const int u = r - kOffW3;
            for(int cc = 0; cc < kBwdCells; cc++) { a = fmaf(X[cc][3], H2[cc][u], a); }
        } else {
            for(int cc = 0; cc < kBwdCells; cc++) { a += X[cc][3]; }
        }
        if(a != 0.0f) { atomicAdd(&grads[r], a); }
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

int cell_features(const pg_particles *p, const pg_cells *cells, const int32_t *perm, int precision, int32_t since,
                  double dt, double half_skin, float *feat, cudaStream_t st) {
    if(!p || !cells || !feat || !p->vel || !p->mass) { return PG_ERR_ARGUMENT; }
    if(precision == PG_MIXED ? !p->force32 : !p->force) { return PG_ERR_ARGUMENT; }
    if(!cells->particle_cell || !cells->cell_count || cells->ncells <= 0) { return PG_ERR_ARGUMENT; }
    const float ts = (float) since, fdt = (float) dt, ihs = (float) (1.0 / half_skin);
    cudaMemsetAsync(feat, 0, (size_t) cells->ncells * kFeat * sizeof(float), st);
    if(p->n > 0) { k_cell_accum<<<blocks_for(p->n), 256, 0, st>>>(*p, *cells, precision, perm, feat); note_launch(); }
    k_cell_finish<<<blocks_for(cells->ncells), 256, 0, st>>>(*cells, ts, fdt, ihs, feat); note_launch();
    return launch_status();
}

int mlp_forward(const float *params, const float *feat, int32_t ncells, float *out, cudaStream_t st) {
    if(!params || !feat || !out || ncells <= 0) { return PG_ERR_ARGUMENT; }
    const int blocks = (int) (((int64_t) ncells * 32 + kFwdThreads - 1) / kFwdThreads);
    k_mlp_forward<<<blocks, kFwdThreads, 0, st>>>(params, feat, ncells, out); note_launch();
    return launch_status();
}

int mlp_softmin(const float *out, int32_t ncells, float temperature, float *result, cudaStream_t st) {
    if(!out || !result || ncells <= 0 || !(temperature > 0.0f)) { return PG_ERR_ARGUMENT; }
    if(ncells <= kSoftminOneBlockMax) {
        k_softmin_block<<<1, kSoftminBlock, 0, st>>>(out, ncells, temperature, result); note_launch();
        return launch_status();
    }
    k_softmin_init<<<1, 1, 0, st>>>(result); note_launch();
    const int blocks = min(blocks_for(ncells), 4 * kSMs);
    k_softmin_min<<<blocks, kBlock, 0, st>>>(out, ncells, reinterpret_cast<int *>(result + 1)); note_launch();
    k_softmin_sum<<<blocks, kBlock, 0, st>>>(out, ncells, 1.0f / temperature, result); note_launch();
    k_softmin_finish<<<1, 1, 0, st>>>(temperature, result); note_launch();
    return launch_status();
}

int cell_select(const float *features, int32_t ncells, int32_t k, float *out, cudaStream_t st) {
    if(!features || !out || k <= 0 || ncells < k) { return PG_ERR_ARGUMENT; }
    k_cell_select<<<k, kSelectThreads, 0, st>>>(features, ncells, k, out); note_launch();
    return launch_status();
}

int mlp_backward(const float *params, const float *feat, const float *out, int32_t ncells, const float *result,
                 float target_log, int censored, float temperature, float *grads, float *loss, cudaStream_t st) {
    if(!params || !feat || !out || !result || !grads || !loss || ncells <= 0) { return PG_ERR_ARGUMENT; }
    const int blocks = (ncells + kBwdCells - 1) / kBwdCells;
    k_mlp_backward<<<blocks, kBwdThreads, 0, st>>>(params, feat, out, ncells, result, target_log, censored,
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
