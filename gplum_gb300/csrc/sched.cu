// Learned work-queue order for the hard part.
//
// The makespan of the persistent hard launch is set by the clusters with the
// longest chains of block steps, and those are not the largest clusters: a
// two-body cluster in a close encounter can take hundreds of block steps.  A
// small FP32 MLP (4 inputs, two hidden layers of 32 tanh units, 1 output)
// predicts log2(1 + block steps) of each cluster from four features the step
// already has, and the hard launch takes its clusters highest prediction
// first.  The model never touches the arithmetic -- any order gives
// bit-identical results -- and without a model the queue is in size order.
//
// Features of a cluster, from the neighbour lists of the last correction:
//   x0 = log2 n                                            (size)
//   x1 = log2 min over neighbour pairs of |dr| / r_out     (closest approach)
//   x2 = log2 (1e-6 + max over pairs of |dv| dt_tree / r_out)  (relative speed)
//   x3 = log2 (dt_tree / min member time step)             (substep estimate)
// (r_out of a pair is the larger of the two.)  Training samples are the
// features of each step's clusters and the block steps the hard launch logged
// for them (p3t_hard_costs).  Training runs on the GPU with this file's own
// kernels: forward, backward (per-tile sums of the per-sample gradients, then
// a fixed-order reduction over tiles, so gradients are deterministic) and
// Adam, on the mean squared error of the standardised target.
#include <algorithm>
#include <cmath>
#include <cstdint>
#include <vector>

#include "../../include/gplum_p3t.h"
#include "p3t_capi_internal.cuh"
#include "p3t_engine.cuh"

namespace p3t {

constexpr int MLP_IN = 4, MLP_H = 32;
constexpr int MLP_NP = MLP_H * MLP_IN + MLP_H + MLP_H * MLP_H + MLP_H + MLP_H + 1;  // 1249
constexpr int MLP_NG = MLP_NP + 1;  // gradients + loss
constexpr int OFF_W1 = 0, OFF_B1 = 128, OFF_W2 = 160, OFF_B2 = 1184, OFF_W3 = 1216, OFF_B3 = 1248;
constexpr int MLP_NORM = 2 * MLP_IN + 2;  // feature mean[4], scale[4], target mean, scale
constexpr int GT = 64;                    // samples per backward tile (= threads per block)

// forward pass of one standardised sample; parameters in shared memory
__device__ __forceinline__ float mlp_forward(const float *P, const float *x, float *h1, float *h2) {
#pragma unroll 4
    for (int i = 0; i < MLP_H; i++) {
        float z = P[OFF_B1 + i];
#pragma unroll
        for (int k = 0; k < MLP_IN; k++) z += P[OFF_W1 + i * MLP_IN + k] * x[k];
        h1[i] = tanhf(z);
    }
    float out = P[OFF_B3];
#pragma unroll 2
    for (int i = 0; i < MLP_H; i++) {
        float z = P[OFF_B2 + i];
#pragma unroll 8
        for (int j = 0; j < MLP_H; j++) z += P[OFF_W2 + i * MLP_H + j] * h1[j];
        h2[i] = tanhf(z);
        out += P[OFF_W3 + i] * h2[i];
    }
    return out;
}

// predictions (denormalised: log2(1 + block steps)) of raw feature rows
__global__ void k_mlp_predict(const float *Pg, const float *norm, const float *X, int n, float *out) {
    __shared__ float P[MLP_NP];
    __shared__ float nm[MLP_NORM];
    for (int i = threadIdx.x; i < MLP_NP; i += blockDim.x) P[i] = Pg[i];
    if (threadIdx.x < MLP_NORM) nm[threadIdx.x] = norm[threadIdx.x];
    __syncthreads();
    const int s = blockIdx.x * blockDim.x + threadIdx.x;
    if (s >= n) return;
    float x[MLP_IN], h1[MLP_H], h2[MLP_H];
#pragma unroll
    for (int k = 0; k < MLP_IN; k++) x[k] = (X[MLP_IN * s + k] - nm[k]) * nm[MLP_IN + k];
    out[s] = mlp_forward(P, x, h1, h2) / nm[2 * MLP_IN + 1] + nm[2 * MLP_IN];
}

// Per-block sums of the per-sample gradients of 0.5 (f(x) - y)^2 (and of the
// loss) over samples idx[b0 .. b0 + nb) of standardised rows Xn, Yn.
// partial[block][MLP_NG].
__global__ void __launch_bounds__(GT) k_mlp_grad(const float *Pg, const float *Xn, const float *Yn, const int *idx,
                                                 int b0, int nb, float *partial) {
    __shared__ float P[MLP_NP];
    __shared__ float xT[MLP_IN][GT], h1T[MLP_H][GT], h2T[MLP_H][GT], dz1T[MLP_H][GT], dz2T[MLP_H][GT];
    __shared__ float d3T[GT], lossT[GT], ones[GT];
    const int t = threadIdx.x;
    for (int i = t; i < MLP_NP; i += GT) P[i] = Pg[i];
    ones[t] = 1.f;
    // the two rows whose dot product is each of this thread's gradient entries
    constexpr int PER = (MLP_NG + GT - 1) / GT;
    const float *ra[PER], *rb[PER];
    float acc[PER];
#pragma unroll
    for (int q = 0; q < PER; q++) {
        const int e = t + q * GT;
        acc[q] = 0.f;
        ra[q] = ones;
        rb[q] = ones;
        if (e < OFF_B1) { ra[q] = dz1T[e / MLP_IN]; rb[q] = xT[e % MLP_IN]; }
        else if (e < OFF_W2) { ra[q] = dz1T[e - OFF_B1]; }
        else if (e < OFF_B2) { ra[q] = dz2T[(e - OFF_W2) / MLP_H]; rb[q] = h1T[(e - OFF_W2) % MLP_H]; }
        else if (e < OFF_W3) { ra[q] = dz2T[e - OFF_B2]; }
        else if (e < OFF_B3) { ra[q] = d3T; rb[q] = h2T[e - OFF_W3]; }
        else if (e == OFF_B3) { ra[q] = d3T; }
        else if (e == MLP_NP) { ra[q] = lossT; }
    }
    __syncthreads();
    const int ntile = (nb + GT - 1) / GT;
    for (int tile = blockIdx.x; tile < ntile; tile += gridDim.x) {
        const int si = tile * GT + t;
        float x[MLP_IN], h1[MLP_H], h2[MLP_H];
        if (si < nb) {
            const int s = idx[b0 + si];
#pragma unroll
            for (int k = 0; k < MLP_IN; k++) x[k] = Xn[MLP_IN * s + k];
            const float e = mlp_forward(P, x, h1, h2) - Yn[s];
            float dz2[MLP_H];
#pragma unroll
            for (int i = 0; i < MLP_H; i++) dz2[i] = e * P[OFF_W3 + i] * (1.f - h2[i] * h2[i]);
#pragma unroll 4
            for (int j = 0; j < MLP_H; j++) {
                float dh = 0.f;
#pragma unroll 8
                for (int i = 0; i < MLP_H; i++) dh += P[OFF_W2 + i * MLP_H + j] * dz2[i];
                dz1T[j][t] = dh * (1.f - h1[j] * h1[j]);
            }
#pragma unroll
            for (int k = 0; k < MLP_IN; k++) xT[k][t] = x[k];
#pragma unroll
            for (int i = 0; i < MLP_H; i++) {
                h1T[i][t] = h1[i];
                h2T[i][t] = h2[i];
                dz2T[i][t] = dz2[i];
            }
            d3T[t] = e;
            lossT[t] = 0.5f * e * e;
        } else {
#pragma unroll
            for (int k = 0; k < MLP_IN; k++) xT[k][t] = 0.f;
#pragma unroll
            for (int i = 0; i < MLP_H; i++) h1T[i][t] = h2T[i][t] = dz1T[i][t] = dz2T[i][t] = 0.f;
            d3T[t] = 0.f;
            lossT[t] = 0.f;
        }
        __syncthreads();
#pragma unroll
        for (int q = 0; q < PER; q++) {
            if (t + q * GT >= MLP_NG) continue;
            float s = 0.f;
            for (int j = 0; j < GT; j++) s += ra[q][j] * rb[q][j];
            acc[q] += s;
        }
        __syncthreads();
    }
#pragma unroll
    for (int q = 0; q < PER; q++)
        if (t + q * GT < MLP_NG) partial[(size_t)blockIdx.x * MLP_NG + t + q * GT] = acc[q];
}

// grad[e] = sum over blocks (fixed order) / n; the loss is accumulated into
// loss_acc when given
__global__ void k_mlp_reduce(const float *partial, int nblk, float inv_n, float *grad, float *loss_acc) {
    const int e = blockIdx.x * blockDim.x + threadIdx.x;
    if (e >= MLP_NG) return;
    float s = 0.f;
    for (int b = 0; b < nblk; b++) s += partial[(size_t)b * MLP_NG + e];
    grad[e] = s * inv_n;
    if (e == MLP_NP && loss_acc) *loss_acc += s * inv_n;
}

__global__ void k_mlp_adam(float *P, const float *g, float *m, float *v, float lr, float b1, float b2, float eps,
                           float c1, float c2) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= MLP_NP) return;
    const float gi = g[i];
    const float mi = b1 * m[i] + (1.f - b1) * gi;
    const float vi = b2 * v[i] + (1.f - b2) * gi * gi;
    m[i] = mi;
    v[i] = vi;
    P[i] -= lr * (mi / c1) / (sqrtf(vi / c2) + eps);
}

// ---- cluster features ---------------------------------------------------------------
__device__ __forceinline__ unsigned fbits(float x) { return __float_as_uint(x); }

__global__ void k_feat_init(int nc, unsigned *red) {
    const int c = blockIdx.x * blockDim.x + threadIdx.x;
    if (c >= nc) return;
    red[3 * c] = fbits(3.0e38f);  // min separation / r_out
    red[3 * c + 1] = 0u;          // max relative speed
    red[3 * c + 2] = fbits(3.0e38f);  // min time step
}

__global__ void k_feat_bodies(State S, const int32_t *cl_of, int cap, double dt_tree, unsigned *red) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= S.n) return;
    const int c = cl_of[i];
    if (c < 0) return;
    const double xi = S.pos[3 * i], yi = S.pos[3 * i + 1], zi = S.pos[3 * i + 2];
    const double ui = S.vel[3 * i], vi = S.vel[3 * i + 1], wi = S.vel[3 * i + 2];
    const double roi = S.r_out_inv[i];
    float sep = 3.0e38f, vr = 0.f;
    const int nn = min(S.nbr_n[i], cap);
    for (int t = 0; t < nn; t++) {
        const int j = S.nbr[(size_t)i * cap + t];
        if (j < 0 || j >= S.n) continue;
        // FP64 differences (positions near 1 AU, separations of 1e-4 AU), the
        // rest in FP32: the features only order the work queue
        const float dx = (float)(S.pos[3 * j] - xi), dy = (float)(S.pos[3 * j + 1] - yi),
                    dz = (float)(S.pos[3 * j + 2] - zi);
        const float du = (float)(S.vel[3 * j] - ui), dv = (float)(S.vel[3 * j + 1] - vi),
                    dw = (float)(S.vel[3 * j + 2] - wi);
        const float r = (float)fmin(roi, S.r_out_inv[j]);
        sep = fminf(sep, sqrtf(dx * dx + dy * dy + dz * dz) * r);
        vr = fmaxf(vr, sqrtf(du * du + dv * dv + dw * dw) * (float)dt_tree * r);
    }
    atomicMin(&red[3 * c], fbits(sep));
    atomicMax(&red[3 * c + 1], fbits(vr));
    atomicMin(&red[3 * c + 2], fbits((float)S.dt[i]));
}

__global__ void k_feat_rows(const unsigned *red, const int32_t *cnt, int nc, float dt_tree, float *X) {
    const int c = blockIdx.x * blockDim.x + threadIdx.x;
    if (c >= nc) return;
    const float sep = __uint_as_float(red[3 * c]), vr = __uint_as_float(red[3 * c + 1]),
                dt = __uint_as_float(red[3 * c + 2]);
    X[4 * c] = log2f((float)max(cnt[c], 1));
    X[4 * c + 1] = log2f(fminf(fmaxf(sep, 1.e-6f), 1.e6f));
    X[4 * c + 2] = log2f(1.e-6f + fminf(vr, 1.e6f));
    X[4 * c + 3] = log2f(dt_tree / fminf(fmaxf(dt, 1.e-30f), 1.e30f));
}

// ---- model state ------------------------------------------------------------------
struct Sched {
    int mode = 0;  // 0 size order, 1 learned
    bool ready = false;
    std::vector<float> params = std::vector<float>(MLP_NP, 0.f), norm = std::vector<float>(MLP_NORM, 0.f);
    DevBuf<float> P, norm_d, g, m, v, partial, X, Xn, Yn, pred, loss;
    DevBuf<unsigned> red;
    DevBuf<int> idx;
    int upload(Context *c) {
        int r = 0;
        if ((r = P.reserve(MLP_NP)) || (r = norm_d.reserve(MLP_NORM))) return r;
        if ((r = h2d(c, P.p, params.data(), MLP_NP * sizeof(float)))) return r;
        return h2d(c, norm_d.p, norm.data(), MLP_NORM * sizeof(float));
    }
};
static Sched g_sched;

static int feature_rows(Context *c, int nc, float *X) {
    Engine &E = g_eng;
    Sched &M = g_sched;
    int r = 0;
    if ((r = M.red.reserve(3 * (size_t)nc + 3))) return r;
    { P3T_COUNT_LAUNCH(); k_feat_init<<<(nc + 255) / 256, 256, 0, c->stream>>>(nc, M.red.p); }
    if (E.S.n > 0)
        { P3T_COUNT_LAUNCH(); k_feat_bodies<<<(E.S.n + 255) / 256, 256, 0, c->stream>>>(E.S, E.cl_of.p, E.cand_cap_alloc,
                                                                    E.params().dt_tree, M.red.p); }
    { P3T_COUNT_LAUNCH(); k_feat_rows<<<(nc + 255) / 256, 256, 0, c->stream>>>(M.red.p, E.cl_cnt.p, nc, (float)E.params().dt_tree, X); }
    return cuda_status(cudaGetLastError());
}

// device priorities of the current clusters for the hard launch's order, or
// nullptr for size order
const float *sched_priority(Context *c, int nc, float *pmin, float *pscale) {
    Sched &M = g_sched;
    if (M.mode != 1 || !M.ready || nc <= 0) return nullptr;
    if (M.X.reserve(4 * (size_t)nc) || M.pred.reserve(nc)) return nullptr;
    if (feature_rows(c, nc, M.X.p)) return nullptr;
    { P3T_COUNT_LAUNCH(); k_mlp_predict<<<(nc + 127) / 128, 128, 0, c->stream>>>(M.P.p, M.norm_d.p, M.X.p, nc, M.pred.p); }
    if (cudaGetLastError() != cudaSuccess) return nullptr;
    *pmin = 0.f;  // predictions are log2(1 + block steps): 1/256 resolution
    *pscale = 256.f;
    return M.pred.p;
}

// standardisation of the training rows: feature mean/scale, target mean/scale
static void fit_norm(const float *x, const float *y, int n, std::vector<float> &norm) {
    for (int k = 0; k < MLP_IN; k++) {
        double s = 0., s2 = 0.;
        for (int i = 0; i < n; i++) {
            s += x[MLP_IN * i + k];
            s2 += (double)x[MLP_IN * i + k] * x[MLP_IN * i + k];
        }
        const double mu = s / n, var = std::max(s2 / n - mu * mu, 1e-12);
        norm[k] = (float)mu;
        norm[MLP_IN + k] = (float)(1.0 / std::sqrt(var));
    }
    double s = 0., s2 = 0.;
    for (int i = 0; i < n; i++) {
        s += y[i];
        s2 += (double)y[i] * y[i];
    }
    const double mu = s / n, var = std::max(s2 / n - mu * mu, 1e-12);
    norm[2 * MLP_IN] = (float)mu;
    norm[2 * MLP_IN + 1] = (float)(1.0 / std::sqrt(var));
}

static int upload_rows(Context *c, const float *x, const float *y, int n) {
    Sched &M = g_sched;
    std::vector<float> xn((size_t)MLP_IN * n), yn(n);
    for (int i = 0; i < n; i++) {
        for (int k = 0; k < MLP_IN; k++)
            xn[(size_t)MLP_IN * i + k] = (x[(size_t)MLP_IN * i + k] - M.norm[k]) * M.norm[MLP_IN + k];
        yn[i] = (y[i] - M.norm[2 * MLP_IN]) * M.norm[2 * MLP_IN + 1];
    }
    int r = 0;
    if ((r = M.Xn.reserve((size_t)MLP_IN * n)) || (r = M.Yn.reserve(n)) || (r = M.idx.reserve(n))) return r;
    if ((r = h2d(c, M.Xn.p, xn.data(), xn.size() * sizeof(float))) || (r = h2d(c, M.Yn.p, yn.data(), n * sizeof(float))))
        return r;
    return 0;
}

static int grad_launch(Context *c, int b0, int nb, const int *idx_dev, float *loss_acc) {
    Sched &M = g_sched;
    int sms = 152;
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, c->device);
    const int nblk = std::max(1, std::min((nb + GT - 1) / GT, sms * 4));
    int r = 0;
    if ((r = M.partial.reserve((size_t)nblk * MLP_NG)) || (r = M.g.reserve(MLP_NG))) return r;
    { P3T_COUNT_LAUNCH(); k_mlp_grad<<<nblk, GT, 0, c->stream>>>(M.P.p, M.Xn.p, M.Yn.p, idx_dev, b0, nb, M.partial.p); }
    { P3T_COUNT_LAUNCH(); k_mlp_reduce<<<(MLP_NG + 255) / 256, 256, 0, c->stream>>>(M.partial.p, nblk, 1.f / (float)nb, M.g.p, loss_acc); }
    return cuda_status(cudaGetLastError());
}

// splitmix64, for the initial weights and the epoch shuffles
static uint64_t splitmix(uint64_t &s) {
    uint64_t z = (s += 0x9e3779b97f4a7c15ULL);
    z = (z ^ (z >> 30)) * 0xbf58476d1ce4e5b9ULL;
    z = (z ^ (z >> 27)) * 0x94d049bb133111ebULL;
    return z ^ (z >> 31);
}

}  // namespace p3t

using namespace p3t;

extern "C" {

int p3t_mlp_set(const float *params, const float *norm) {
    Context *c = ctx_get(0);
    if (!c) return -(int)cudaErrorNoDevice;
    Sched &M = g_sched;
    M.params.assign(params, params + MLP_NP);
    M.norm.assign(norm, norm + MLP_NORM);
    int r = M.upload(c);
    if (r) return r;
    M.ready = true;
    return cuda_status(cudaStreamSynchronize(c->stream));
}

int p3t_mlp_get(float *params, float *norm) {
    Context *c = ctx_get(0);
    if (!c) return -(int)cudaErrorNoDevice;
    Sched &M = g_sched;
    if (M.ready && M.P.p) {
        int r = d2h(c, M.params.data(), M.P.p, MLP_NP * sizeof(float));
        if (r) return r;
    }
    std::copy(M.params.begin(), M.params.end(), params);
    std::copy(M.norm.begin(), M.norm.end(), norm);
    return M.ready ? 0 : ST_BAD_INDEX;
}

int p3t_mlp_predict(const float *x, int n, float *out) {
    Context *c = ctx_get(0);
    if (!c) return -(int)cudaErrorNoDevice;
    Sched &M = g_sched;
    if (!M.ready || n < 0) return ST_BAD_INDEX;
    if (n == 0) return 0;
    int r = 0;
    if ((r = M.X.reserve(4 * (size_t)n)) || (r = M.pred.reserve(n))) return r;
    if ((r = h2d(c, M.X.p, x, 4 * (size_t)n * sizeof(float)))) return r;
    { P3T_COUNT_LAUNCH(); k_mlp_predict<<<(n + 127) / 128, 128, 0, c->stream>>>(M.P.p, M.norm_d.p, M.X.p, n, M.pred.p); }
    if ((r = cuda_status(cudaGetLastError()))) return r;
    return d2h(c, out, M.pred.p, n * sizeof(float));
}

int p3t_mlp_loss_grad(const float *x, const float *y, int n, float *loss, float *grad) {
    Context *c = ctx_get(0);
    if (!c) return -(int)cudaErrorNoDevice;
    Sched &M = g_sched;
    if (!M.ready || n <= 0) return ST_BAD_INDEX;
    int r = 0;
    if ((r = upload_rows(c, x, y, n))) return r;
    std::vector<int> id(n);
    for (int i = 0; i < n; i++) id[i] = i;
    if ((r = h2d(c, M.idx.p, id.data(), n * sizeof(int)))) return r;
    if ((r = grad_launch(c, 0, n, M.idx.p, nullptr))) return r;
    std::vector<float> g(MLP_NG);
    if ((r = d2h(c, g.data(), M.g.p, MLP_NG * sizeof(float)))) return r;
    std::copy(g.begin(), g.begin() + MLP_NP, grad);
    *loss = g[MLP_NP];
    return 0;
}

int p3t_mlp_train(const float *x, const float *y, int n, int epochs, int batch, float lr, unsigned long long seed,
                  float *loss_per_epoch) {
    Context *c = ctx_get(0);
    if (!c) return -(int)cudaErrorNoDevice;
    Sched &M = g_sched;
    if (n <= 0 || epochs < 0 || batch <= 0) return ST_BAD_INDEX;
    uint64_t s = seed;
    if (!M.ready) {
        // uniform initial weights in +-sqrt(6 / (fan_in + fan_out)), zero biases
        auto fill = [&](int off, int cnt, int fin, int fout) {
            const double a = std::sqrt(6.0 / (fin + fout));
            for (int i = 0; i < cnt; i++) M.params[off + i] = (float)(a * (2.0 * ((splitmix(s) >> 11) * 0x1.0p-53) - 1.0));
        };
        std::fill(M.params.begin(), M.params.end(), 0.f);
        fill(OFF_W1, MLP_H * MLP_IN, MLP_IN, MLP_H);
        fill(OFF_W2, MLP_H * MLP_H, MLP_H, MLP_H);
        fill(OFF_W3, MLP_H, MLP_H, 1);
        fit_norm(x, y, n, M.norm);
        int r = M.upload(c);
        if (r) return r;
        M.ready = true;
    }
    int r = 0;
    if ((r = upload_rows(c, x, y, n)) || (r = M.m.reserve(MLP_NP)) || (r = M.v.reserve(MLP_NP)) ||
        (r = M.loss.reserve(1)))
        return r;
    cudaMemsetAsync(M.m.p, 0, MLP_NP * sizeof(float), c->stream);
    cudaMemsetAsync(M.v.p, 0, MLP_NP * sizeof(float), c->stream);
    std::vector<int> perm(n);
    for (int i = 0; i < n; i++) perm[i] = i;
    const float b1 = 0.9f, b2 = 0.999f;
    double p1 = 1., p2 = 1.;
    const int nbatch = (n + batch - 1) / batch;
    for (int ep = 0; ep < epochs; ep++) {
        for (int i = n - 1; i > 0; i--) std::swap(perm[i], perm[(int)(splitmix(s) % (uint64_t)(i + 1))]);
        if ((r = h2d(c, M.idx.p, perm.data(), n * sizeof(int)))) return r;
        cudaMemsetAsync(M.loss.p, 0, sizeof(float), c->stream);
        for (int b = 0; b < nbatch; b++) {
            const int b0 = b * batch, nb = std::min(batch, n - b0);
            if ((r = grad_launch(c, b0, nb, M.idx.p, M.loss.p))) return r;
            p1 *= b1;
            p2 *= b2;
            { P3T_COUNT_LAUNCH(); k_mlp_adam<<<(MLP_NP + 255) / 256, 256, 0, c->stream>>>(M.P.p, M.g.p, M.m.p, M.v.p, lr, b1, b2, 1e-8f,
                                                                      (float)(1. - p1), (float)(1. - p2)); }
        }
        float l = 0.f;
        if ((r = cuda_status(cudaMemcpyAsync(&l, M.loss.p, sizeof(float), cudaMemcpyDeviceToHost, c->stream))) ||
            (r = cuda_status(cudaStreamSynchronize(c->stream))))
            return r;
        if (loss_per_epoch) loss_per_epoch[ep] = l / nbatch;
    }
    return d2h(c, M.params.data(), M.P.p, MLP_NP * sizeof(float));
}

int p3t_mlp_reset(void) {
    g_sched.ready = false;
    return 0;
}

int p3t_cluster_features(float *out, int n) {
    Engine &E = g_eng;
    if (!E.c) return -(int)cudaErrorNoDevice;
    if (n != E.n_clusters) return ST_BAD_INDEX;
    if (n == 0) return 0;
    Sched &M = g_sched;
    int r = 0;
    if ((r = M.X.reserve(4 * (size_t)n)) || (r = feature_rows(E.c, n, M.X.p))) return r;
    return d2h(E.c, out, M.X.p, 4 * (size_t)n * sizeof(float));
}

int p3t_set_schedule(int mode) {
    if (mode != 0 && mode != 1) return ST_BAD_INDEX;
    g_sched.mode = mode;
    return 0;
}

}  // extern "C"
