// Learned preconditioner correction: a 3-layer message-passing network (hidden width 64) on the
// node graph of the 3x3-block system, with hand-written forward, backward and Adam kernels.
//
// Per node m (3 DOFs) the input features are f_m = [s0 * (Mv)_m, s1 * v_m, s2 * (D^-1 v)_m]
// (9 values; Mv is the multigrid V-cycle applied to v, D^-1 the block-Jacobi inverse, s fixed
// scales).  With row-normalised coupling weights a_mn = |A_mn|_F / sum_{n'!=m} |A_mn'|_F:
//   h0   = relu(W_in f)
//   for l = 1..3:  agg_l[m] = sum_{n != m} a_mn h_{l-1}[n]
//                  q_l = relu(Ws_l h_{l-1} + Wn_l agg_l),   h_l = h_{l-1} + q_l
//   out  = W_out h3 (3 per node),   z = Mv + out   (Dirichlet DOFs -> 0)
// No biases: the network is positively homogeneous (z(alpha v) = alpha z(v), alpha > 0), so the
// FGMRES basis vectors need no normalisation.  Weights are stored in BF16 for inference and
// kept as FP32 masters for training; all accumulation is FP32.  Weight-gradient reductions are
// per-CTA partials summed in a fixed order (deterministic).

#include <cuda_bf16.h>

#include "ef_common.cuh"

namespace ef {

constexpr int H = 64;    // hidden width
constexpr int FIN = 9;   // input features per node
constexpr int NL = 3;    // message-passing layers
constexpr int TILE = 64; // nodes per CTA tile in the dense layers

// parameter layout (floats): W_in [H][FIN], then per layer Ws [H][H], Wn [H][H], then W_out [3][H]
constexpr int OFF_WIN = 0;
constexpr int OFF_L0 = H * FIN;
constexpr int PER_LAYER = 2 * H * H;
constexpr int OFF_WOUT = OFF_L0 + NL * PER_LAYER;
constexpr int NPARAM = OFF_WOUT + 3 * H;

// coupling weights a (row-normalised Frobenius norms, self block 0) and the transposed weights
// aT[(m,k)] = a[(k,m)] used by the backward aggregation
__global__ void edge_weight_kernel(int nN, const int32_t* __restrict__ rowPtr, const int32_t* __restrict__ colIdx,
                                   const float* __restrict__ vals, float* __restrict__ a) {
    const int m = blockIdx.x * blockDim.x + threadIdx.x;
    if (m >= nN) return;
    float tot = 0.f;
    for (int k = rowPtr[m]; k < rowPtr[m + 1]; ++k) {
        if (colIdx[k] == m) continue;
        const float* v = vals + (int64_t)k * 9;
        float s = 0.f;
        for (int i = 0; i < 9; ++i) s += v[i] * v[i];
        tot += sqrtf(s);
    }
    const float inv = tot > 0.f ? 1.f / tot : 0.f;
    for (int k = rowPtr[m]; k < rowPtr[m + 1]; ++k) {
        if (colIdx[k] == m) {
            a[k] = 0.f;
            continue;
        }
        const float* v = vals + (int64_t)k * 9;
        float s = 0.f;
        for (int i = 0; i < 9; ++i) s += v[i] * v[i];
        a[k] = sqrtf(s) * inv;
    }
}

__global__ void gather_kernel(int64_t n, const int64_t* __restrict__ idx, const float* __restrict__ src,
                              float* __restrict__ dst) {
    const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) dst[i] = src[idx[i]];
}

// f[m] = [s0 * Mv_m, s1 * v_m, s2 * (D^-1 v)_m]
__global__ void features_kernel(int nN, const float* __restrict__ Mv, const float* __restrict__ v,
                                const float* __restrict__ binv, float s0, float s1, float s2, float* __restrict__ f) {
    const int m = blockIdx.x * blockDim.x + threadIdx.x;
    if (m >= nN) return;
    const float v0 = v[3 * m], v1 = v[3 * m + 1], v2 = v[3 * m + 2];
    const float* B = binv + (int64_t)m * 9;
    float* o = f + (int64_t)m * FIN;
#pragma unroll
    for (int i = 0; i < 3; ++i) {
        o[i] = s0 * Mv[3 * m + i];
        o[3 + i] = s1 * v[3 * m + i];
        o[6 + i] = s2 * (B[3 * i] * v0 + B[3 * i + 1] * v1 + B[3 * i + 2] * v2);
    }
}

// h0 = relu(W_in f); one thread per (node, channel)
__global__ void input_kernel(int nN, const float* __restrict__ f, const float* __restrict__ P,
                             float* __restrict__ h0) {
    const int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= (int64_t)nN * H) return;
    const int m = (int)(t / H), c = (int)(t % H);
    const float* w = P + OFF_WIN + c * FIN;
    const float* x = f + (int64_t)m * FIN;
    float s = 0.f;
#pragma unroll
    for (int j = 0; j < FIN; ++j) s += w[j] * x[j];
    h0[t] = fmaxf(s, 0.f);
}

// agg[m] = sum_k w[k] h[col[k]] over the block row of m; one warp per node, 2 channels per lane
__global__ void aggregate_kernel(int nN, const int32_t* __restrict__ rowPtr, const int32_t* __restrict__ colIdx,
                                 const float* __restrict__ w, const float* __restrict__ h, float* __restrict__ agg,
                                 int accumulate) {
    const int lane = threadIdx.x & 31;
    const int m = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    if (m >= nN) return;
    float a0 = 0.f, a1 = 0.f;
    for (int k = rowPtr[m]; k < rowPtr[m + 1]; ++k) {
        const float wk = w[k];
        if (wk == 0.f) continue;
        const float* hn = h + (int64_t)colIdx[k] * H;
        a0 += wk * hn[lane];
        a1 += wk * hn[lane + 32];
    }
    float* o = agg + (int64_t)m * H;
    if (accumulate) {
        o[lane] += a0;
        o[lane + 32] += a1;
    } else {
        o[lane] = a0;
        o[lane + 32] = a1;
    }
}

// dense layer: q = relu(Ws h + Wn agg), hout = h + q; 64-node tiles, weights in shared memory
__global__ void __launch_bounds__(256) dense_kernel(int nN, const float* __restrict__ h, const float* __restrict__ agg,
                                                    const float* __restrict__ Wl, float* __restrict__ q,
                                                    float* __restrict__ hout) {
    extern __shared__ float dsm[];
    float(*Ws)[H + 1] = reinterpret_cast<float(*)[H + 1]>(dsm);
    float(*Wn)[H + 1] = Ws + H;
    float(*xs)[H + 1] = Wn + H;
    float(*as)[H + 1] = xs + TILE;
    for (int i = threadIdx.x; i < H * H; i += blockDim.x) {
        Ws[i / H][i % H] = Wl[i];
        Wn[i / H][i % H] = Wl[H * H + i];
    }
    const int m0 = blockIdx.x * TILE;
    for (int i = threadIdx.x; i < TILE * H; i += blockDim.x) {
        const int r = i / H, c = i % H;
        const bool ok = m0 + r < nN;
        xs[r][c] = ok ? h[(int64_t)(m0 + r) * H + c] : 0.f;
        as[r][c] = ok ? agg[(int64_t)(m0 + r) * H + c] : 0.f;
    }
    __syncthreads();
    // thread -> 4 nodes x 4 channels
    const int tc = threadIdx.x % 16, tr = threadIdx.x / 16;
    float acc[4][4];
#pragma unroll
    for (int i = 0; i < 4; ++i)
#pragma unroll
        for (int j = 0; j < 4; ++j) acc[i][j] = 0.f;
    for (int k = 0; k < H; ++k) {
        float xa[4], aa[4], ws[4], wn[4];
#pragma unroll
        for (int i = 0; i < 4; ++i) {
            xa[i] = xs[tr * 4 + i][k];
            aa[i] = as[tr * 4 + i][k];
        }
#pragma unroll
        for (int j = 0; j < 4; ++j) {
            ws[j] = Ws[tc * 4 + j][k];
            wn[j] = Wn[tc * 4 + j][k];
        }
#pragma unroll
        for (int i = 0; i < 4; ++i)
#pragma unroll
            for (int j = 0; j < 4; ++j) acc[i][j] += ws[j] * xa[i] + wn[j] * aa[i];
    }
#pragma unroll
    for (int i = 0; i < 4; ++i) {
        const int m = m0 + tr * 4 + i;
        if (m >= nN) continue;
#pragma unroll
        for (int j = 0; j < 4; ++j) {
            const int c = tc * 4 + j;
            const float qq = fmaxf(acc[i][j], 0.f);
            q[(int64_t)m * H + c] = qq;
            hout[(int64_t)m * H + c] = xs[tr * 4 + i][c] + qq;
        }
    }
}

// z = base + so * W_out h3 on free DOFs (0 on masked); base may be null
__global__ void output_kernel(int nN, const float* __restrict__ h3, const float* __restrict__ P,
                              const float* __restrict__ base, const uint8_t* __restrict__ mask, float so,
                              float* __restrict__ z) {
    const int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= (int64_t)nN * 3) return;
    const int m = (int)(t / 3), c = (int)(t % 3);
    const float* w = P + OFF_WOUT + c * H;
    const float* x = h3 + (int64_t)m * H;
    float s = 0.f;
#pragma unroll 8
    for (int j = 0; j < H; ++j) s += w[j] * x[j];
    const float b = base ? base[t] : 0.f;
    z[t] = (mask && mask[t]) ? 0.f : b + so * s;
}

// ---- backward ------------------------------------------------------------------------------

// dout = so * scale * (z - e) on free DOFs; dh3[m] = W_out^T dout[m]
__global__ void output_backward_kernel(int nN, const float* __restrict__ z, const float* __restrict__ e,
                                       const uint8_t* __restrict__ mask, float scale, float so,
                                       const float* __restrict__ P, float* __restrict__ dout, float* __restrict__ dh3) {
    const int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= (int64_t)nN * H) return;
    const int m = (int)(t / H), c = (int)(t % H);
    float s = 0.f;
#pragma unroll
    for (int i = 0; i < 3; ++i) {
        const int d = 3 * m + i;
        const float g = (mask && mask[d]) ? 0.f : so * scale * (z[d] - (e ? e[d] : 0.f));
        if (c == 0) dout[d] = g;
        s += P[OFF_WOUT + i * H + c] * g;
    }
    dh3[t] = s;
}

// per-CTA partial of G[i][j] = sum_m A[m][i] * B[m][j] (A: [n][ra], B: [n][rb]); grid-stride tiles
__global__ void __launch_bounds__(256) outer_partial_kernel(int n, int ra, int rb, const float* __restrict__ A,
                                                            const float* __restrict__ B, float* __restrict__ part) {
    // each thread owns up to 16 entries (i, j) of the ra x rb result
    const int nEnt = ra * rb;
    float acc[16];
#pragma unroll
    for (int q = 0; q < 16; ++q) acc[q] = 0.f;
    __shared__ float as_[TILE][H + 1], bs_[TILE][H + 1];
    for (int m0 = blockIdx.x * TILE; m0 < n; m0 += gridDim.x * TILE) {
        __syncthreads();
        for (int i = threadIdx.x; i < TILE * H; i += blockDim.x) {
            const int r = i / H, c = i % H;
            const bool ok = m0 + r < n;
            as_[r][c] = (ok && c < ra) ? A[(int64_t)(m0 + r) * ra + c] : 0.f;
            bs_[r][c] = (ok && c < rb) ? B[(int64_t)(m0 + r) * rb + c] : 0.f;
        }
        __syncthreads();
#pragma unroll
        for (int q = 0; q < 16; ++q) {
            const int ent = threadIdx.x + q * 256;
            if (ent >= nEnt) break;
            const int i = ent / rb, j = ent % rb;
            float s = acc[q];
            for (int r = 0; r < TILE; ++r) s += as_[r][i] * bs_[r][j];
            acc[q] = s;
        }
    }
#pragma unroll
    for (int q = 0; q < 16; ++q) {
        const int ent = threadIdx.x + q * 256;
        if (ent < nEnt) part[(int64_t)blockIdx.x * nEnt + ent] = acc[q];
    }
}

// g[ent] = sum over CTAs of part (fixed order)
__global__ void partial_sum_kernel(int nPart, int nEnt, const float* __restrict__ part, float* __restrict__ g) {
    const int ent = blockIdx.x * blockDim.x + threadIdx.x;
    if (ent >= nEnt) return;
    float s = 0.f;
    for (int c = 0; c < nPart; ++c) s += part[(int64_t)c * nEnt + ent];
    g[ent] = s;
}

// du = dh * (q > 0); gs = Ws^T du; gn = Wn^T du; dhprev = dh + gs   (64-node tiles)
__global__ void __launch_bounds__(256) dense_backward_kernel(int nN, const float* __restrict__ dh,
                                                             const float* __restrict__ q, const float* __restrict__ Wl,
                                                             float* __restrict__ du, float* __restrict__ gn,
                                                             float* __restrict__ dhprev) {
    extern __shared__ float dsm[];
    float(*Ws)[H + 1] = reinterpret_cast<float(*)[H + 1]>(dsm);
    float(*Wn)[H + 1] = Ws + H;
    float(*ds)[H + 1] = Wn + H;
    for (int i = threadIdx.x; i < H * H; i += blockDim.x) {
        Ws[i / H][i % H] = Wl[i];
        Wn[i / H][i % H] = Wl[H * H + i];
    }
    const int m0 = blockIdx.x * TILE;
    for (int i = threadIdx.x; i < TILE * H; i += blockDim.x) {
        const int r = i / H, c = i % H;
        const int64_t g = (int64_t)(m0 + r) * H + c;
        float d = 0.f;
        if (m0 + r < nN) {
            d = q[g] > 0.f ? dh[g] : 0.f;
            du[g] = d;
        }
        ds[r][c] = d;
    }
    __syncthreads();
    const int tc = threadIdx.x % 16, tr = threadIdx.x / 16;
    float as_[4][4], an[4][4];
#pragma unroll
    for (int i = 0; i < 4; ++i)
#pragma unroll
        for (int j = 0; j < 4; ++j) as_[i][j] = an[i][j] = 0.f;
    for (int k = 0; k < H; ++k) {  // gs[m][c] = sum_k Ws[k][c] du[m][k]
        float dd[4], ws[4], wn[4];
#pragma unroll
        for (int i = 0; i < 4; ++i) dd[i] = ds[tr * 4 + i][k];
#pragma unroll
        for (int j = 0; j < 4; ++j) {
            ws[j] = Ws[k][tc * 4 + j];
            wn[j] = Wn[k][tc * 4 + j];
        }
#pragma unroll
        for (int i = 0; i < 4; ++i)
#pragma unroll
            for (int j = 0; j < 4; ++j) {
                as_[i][j] += ws[j] * dd[i];
                an[i][j] += wn[j] * dd[i];
            }
    }
#pragma unroll
    for (int i = 0; i < 4; ++i) {
        const int m = m0 + tr * 4 + i;
        if (m >= nN) continue;
#pragma unroll
        for (int j = 0; j < 4; ++j) {
            const int64_t g = (int64_t)m * H + tc * 4 + j;
            dhprev[g] = dh[g] + as_[i][j];
            gn[g] = an[i][j];
        }
    }
}

// du0 = dh0 * (h0 > 0)
__global__ void relu_mask_kernel(int64_t n, const float* __restrict__ dh, const float* __restrict__ hact,
                                 float* __restrict__ d) {
    const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) d[i] = hact[i] > 0.f ? dh[i] : 0.f;
}

// Adam step on FP32 masters, refreshes the BF16 inference copy and the FP32 view of it
__global__ void adam_kernel(int n, float* __restrict__ p, const float* __restrict__ g, float* __restrict__ m1,
                            float* __restrict__ m2, float lr, float b1, float b2, float eps, float c1, float c2,
                            __nv_bfloat16* __restrict__ pb, float* __restrict__ pf) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const float gi = g[i];
    const float a = b1 * m1[i] + (1.f - b1) * gi;
    const float b = b2 * m2[i] + (1.f - b2) * gi * gi;
    m1[i] = a;
    m2[i] = b;
    const float upd = lr * (a / c1) / (sqrtf(b / c2) + eps);
    const float np = p[i] - upd;
    p[i] = np;
    const __nv_bfloat16 q = __float2bfloat16(np);
    pb[i] = q;
    pf[i] = __bfloat162float(q);
}

// BF16 inference copy and its FP32 view from the FP32 masters
__global__ void refresh_kernel(int n, const float* __restrict__ p, __nv_bfloat16* __restrict__ pb,
                               float* __restrict__ pf) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const __nv_bfloat16 q = __float2bfloat16(p[i]);
    pb[i] = q;
    pf[i] = __bfloat162float(q);
}

__global__ void bf16_to_f32_kernel(int n, const __nv_bfloat16* __restrict__ pb, float* __restrict__ pf) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) pf[i] = __bfloat162float(pb[i]);
}

// per-CTA partial sums in FP64 over the free DOFs: mode 1: (z - e)^2 (e may be null: z^2);
// mode 0: z . e; mode 3: z^2 per 3-wide feature group of f ([n][9], no mask)
__global__ void sumsq_partial_kernel(int64_t n, int groups, const float* __restrict__ z, const float* __restrict__ e,
                                     const uint8_t* __restrict__ mask, double* __restrict__ part) {
    __shared__ double red[8][3];
    double acc[3] = {0.0, 0.0, 0.0};
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
        if (groups == 0) {
            if (mask && mask[i]) continue;
            acc[0] += (double)z[i] * (double)e[i];
        } else if (groups == 3) {
            const int g = (int)((i % FIN) / 3);
            const double v = z[i];
            acc[0] += g == 0 ? v * v : 0.0;
            acc[1] += g == 1 ? v * v : 0.0;
            acc[2] += g == 2 ? v * v : 0.0;
        } else {
            if (mask && mask[i]) continue;
            const double d = (double)z[i] - (e ? (double)e[i] : 0.0);
            acc[0] += d * d;
        }
    }
    const int lane = threadIdx.x & 31, wp = threadIdx.x >> 5;
#pragma unroll
    for (int g = 0; g < 3; ++g) {
        double a = acc[g];
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) a += __shfl_xor_sync(0xffffffffu, a, o);
        if (lane == 0) red[wp][g] = a;
    }
    __syncthreads();
    if (threadIdx.x < 3) {
        double t = 0.0;
        for (int w = 0; w < (int)(blockDim.x >> 5); ++w) t += red[w][threadIdx.x];
        part[(int64_t)blockIdx.x * 3 + threadIdx.x] = t;
    }
}

__global__ void sumsq_final_kernel(int nPart, const double* __restrict__ part, double* __restrict__ out) {
    const int g = threadIdx.x;
    if (g >= 3) return;
    double t = 0.0;
    for (int c = 0; c < nPart; ++c) t += part[(int64_t)c * 3 + g];
    out[g] = t;
}

__global__ void scale_inplace_kernel(int64_t n, float* __restrict__ x, float a) {
    const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) x[i] *= a;
}

// fs[m][i] = s[i / 3] * f[m][i]
__global__ void scale_features_kernel(int64_t n, const float* __restrict__ f, float s0, float s1, float s2,
                                      float* __restrict__ fs) {
    const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const int g = (int)((i % FIN) / 3);
    fs[i] = f[i] * (g == 0 ? s0 : (g == 1 ? s1 : s2));
}

// z = Mv + alpha N on free DOFs (0 on masked), alpha = dots[0] / dots[3] (0 if dots[3] <= 0):
// the step length along the network output that minimises |v - K z| given rho.KN and |KN|^2
__global__ void alpha_combine_kernel(int64_t n, const float* __restrict__ Mv, const float* __restrict__ N,
                                     const double* __restrict__ dots, const uint8_t* __restrict__ mask,
                                     float* __restrict__ z) {
    const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const double den = dots[3];
    const float alpha = den > 0.0 ? (float)(dots[0] / den) : 0.f;
    z[i] = (mask && mask[i]) ? 0.f : Mv[i] + alpha * N[i];
}

}  // namespace ef

using namespace ef;

static inline int nbm(int64_t n, int t) { return (int)((n + t - 1) / t); }
static const size_t kDenseSmem = sizeof(float) * (2 * H + 2 * TILE) * (H + 1);
static const size_t kDenseBwdSmem = sizeof(float) * (2 * H + TILE) * (H + 1);

ef_status ef_mpnn_setup_kernels() {
    EF_CUDA(cudaFuncSetAttribute(dense_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)kDenseSmem));
    EF_CUDA(cudaFuncSetAttribute(dense_backward_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)kDenseBwdSmem));
    return EF_OK;
}

int ef_mpnn_nparam() { return NPARAM; }
int ef_mpnn_hidden() { return H; }
int ef_mpnn_layer_offset(int l) { return OFF_L0 + l * PER_LAYER; }
int ef_mpnn_out_offset() { return OFF_WOUT; }

ef_status ef_launch_edge_weights(int nN, const int32_t* rowPtr, const int32_t* colIdx, const float* vals, float* a,
                                 cudaStream_t s) {
    edge_weight_kernel<<<nbm(nN, 128), 128, 0, ef::counted(s)>>>(nN, rowPtr, colIdx, vals, a);
    EF_CUDA(cudaGetLastError());
    return EF_OK;
}

ef_status ef_launch_gather_f32(int64_t n, const int64_t* idx, const float* src, float* dst, cudaStream_t s) {
    if (n == 0) return EF_OK;
    gather_kernel<<<nbm(n, 256), 256, 0, ef::counted(s)>>>(n, idx, src, dst);
    EF_CUDA(cudaGetLastError());
    return EF_OK;
}

// forward pass; acts = [h0 | q1 h1 agg1 | q2 h2 agg2 | q3 h3 agg3] (each nN x H floats)
ef_status ef_mpnn_forward(int nN, const int32_t* rowPtr, const int32_t* colIdx, const float* a, const float* P,
                          const float* f, const float* base, const uint8_t* mask, float so, float* acts, float* z,
                          cudaStream_t s) {
    const int64_t NH = (int64_t)nN * H;
    float* h0 = acts;
    input_kernel<<<nbm(NH, 256), 256, 0, ef::counted(s)>>>(nN, f, P, h0);
    const float* hprev = h0;
    for (int l = 0; l < NL; ++l) {
        float* q = acts + NH * (1 + 3 * l);
        float* hl = q + NH;
        float* agg = hl + NH;
        aggregate_kernel<<<nbm((int64_t)nN * 32, 256), 256, 0, ef::counted(s)>>>(nN, rowPtr, colIdx, a, hprev, agg, 0);
        dense_kernel<<<nbm(nN, TILE), 256, kDenseSmem, ef::counted(s)>>>(nN, hprev, agg, P + OFF_L0 + l * PER_LAYER, q, hl);
        hprev = hl;
    }
    output_kernel<<<nbm((int64_t)nN * 3, 256), 256, 0, ef::counted(s)>>>(nN, hprev, P, base, mask, so, z);
    EF_CUDA(cudaGetLastError());
    return EF_OK;
}

// backward pass for loss L = 0.5 * scale * sum_free (z - e)^2 (scale folds the 1/|e|^2 factor and 2);
// grad [NPARAM] overwritten; work: 4 x nN x H floats; part: nPart x H*H floats
ef_status ef_mpnn_backward(int nN, const int32_t* rowPtr, const int32_t* colIdx, const float* aT, const float* P,
                           const float* f, const float* acts, const float* z, const float* e, const uint8_t* mask,
                           float scale, float so, float* grad, float* work, float* part, int nPart, cudaStream_t s) {
    const int64_t NH = (int64_t)nN * H;
    float* dh = work;
    float* du = work + NH;
    float* gn = work + 2 * NH;
    float* dout = part;  // [3 nN] before the partials are needed
    const float* h0 = acts;
    const float* h3 = acts + NH * (1 + 3 * (NL - 1)) + NH;
    // output layer: dh3 and grad W_out = dout^T h3
    float* doutBuf = gn;  // reuse gn storage for dout (3 nN <= nN H)
    (void)dout;
    output_backward_kernel<<<nbm(NH, 256), 256, 0, ef::counted(s)>>>(nN, z, e, mask, scale, so, P, doutBuf, dh);
    outer_partial_kernel<<<nPart, 256, 0, ef::counted(s)>>>(nN, 3, H, doutBuf, h3, part);
    partial_sum_kernel<<<nbm(3 * H, 256), 256, 0, ef::counted(s)>>>(nPart, 3 * H, part, grad + OFF_WOUT);
    for (int l = NL - 1; l >= 0; --l) {
        const float* q = acts + NH * (1 + 3 * l);
        const float* agg = q + 2 * NH;
        const float* hprev = l == 0 ? h0 : acts + NH * (1 + 3 * (l - 1)) + NH;
        // du, gn, dhprev (written into dh in place is unsafe: use du as temp for dhprev afterwards)
        float* dhprev = work + 3 * NH;
        dense_backward_kernel<<<nbm(nN, TILE), 256, kDenseBwdSmem, ef::counted(s)>>>(nN, dh, q, P + OFF_L0 + l * PER_LAYER, du, gn,
                                                                         dhprev);
        // grads Ws_l = du^T hprev, Wn_l = du^T agg
        outer_partial_kernel<<<nPart, 256, 0, ef::counted(s)>>>(nN, H, H, du, hprev, part);
        partial_sum_kernel<<<nbm(H * H, 256), 256, 0, ef::counted(s)>>>(nPart, H * H, part, grad + OFF_L0 + l * PER_LAYER);
        outer_partial_kernel<<<nPart, 256, 0, ef::counted(s)>>>(nN, H, H, du, agg, part);
        partial_sum_kernel<<<nbm(H * H, 256), 256, 0, ef::counted(s)>>>(nPart, H * H, part, grad + OFF_L0 + l * PER_LAYER + H * H);
        // transpose aggregation: dhprev[m] += sum_k aT[(m,k)] gn[k]
        aggregate_kernel<<<nbm((int64_t)nN * 32, 256), 256, 0, ef::counted(s)>>>(nN, rowPtr, colIdx, aT, gn, dhprev, 1);
        EF_CUDA(cudaMemcpyAsync(dh, dhprev, sizeof(float) * NH, cudaMemcpyDeviceToDevice, s));
    }
    // input layer: grad W_in = (dh0 * relu'(h0))^T f
    relu_mask_kernel<<<nbm(NH, 256), 256, 0, ef::counted(s)>>>(NH, dh, h0, du);
    outer_partial_kernel<<<nPart, 256, 0, ef::counted(s)>>>(nN, H, FIN, du, f, part);
    partial_sum_kernel<<<nbm(H * FIN, 256), 256, 0, ef::counted(s)>>>(nPart, H * FIN, part, grad + OFF_WIN);
    EF_CUDA(cudaGetLastError());
    return EF_OK;
}

ef_status ef_mpnn_adam(int n, float* p, const float* g, float* m1, float* m2, float lr, float b1, float b2, float eps,
                       int step, void* pb, float* pf, cudaStream_t s) {
    const float c1 = 1.f - powf(b1, (float)step), c2 = 1.f - powf(b2, (float)step);
    adam_kernel<<<nbm(n, 256), 256, 0, ef::counted(s)>>>(n, p, g, m1, m2, lr, b1, b2, eps, c1, c2, (__nv_bfloat16*)pb, pf);
    EF_CUDA(cudaGetLastError());
    return EF_OK;
}

ef_status ef_launch_features(int nN, const float* Mv, const float* v, const float* binv, float s0, float s1, float s2,
                             float* f, cudaStream_t s) {
    features_kernel<<<nbm(nN, 256), 256, 0, ef::counted(s)>>>(nN, Mv, v, binv, s0, s1, s2, f);
    EF_CUDA(cudaGetLastError());
    return EF_OK;
}

ef_status ef_mpnn_bf16_to_f32(int n, const void* pb, float* pf, cudaStream_t s) {
    bf16_to_f32_kernel<<<nbm(n, 256), 256, 0, ef::counted(s)>>>(n, (const __nv_bfloat16*)pb, pf);
    EF_CUDA(cudaGetLastError());
    return EF_OK;
}

// out[0..3) = the sums of sumsq_partial_kernel (mode `groups`); part holds nPart x 3 doubles;
// deterministic
ef_status ef_mpnn_sumsq(int64_t n, int groups, const float* z, const float* e, const uint8_t* mask, double* part,
                        int nPart, double* out, cudaStream_t s) {
    sumsq_partial_kernel<<<nPart, 256, 0, ef::counted(s)>>>(n, groups, z, e, mask, part);
    sumsq_final_kernel<<<1, 32, 0, ef::counted(s)>>>(nPart, part, out);
    EF_CUDA(cudaGetLastError());
    return EF_OK;
}

ef_status ef_mpnn_scale(int64_t n, float* x, float a, cudaStream_t s) {
    if (n == 0) return EF_OK;
    scale_inplace_kernel<<<nbm(n, 256), 256, 0, ef::counted(s)>>>(n, x, a);
    EF_CUDA(cudaGetLastError());
    return EF_OK;
}

ef_status ef_mpnn_scale_features(int nN, const float* f, float s0, float s1, float s2, float* fs, cudaStream_t s) {
    const int64_t n = (int64_t)nN * FIN;
    scale_features_kernel<<<nbm(n, 256), 256, 0, ef::counted(s)>>>(n, f, s0, s1, s2, fs);
    EF_CUDA(cudaGetLastError());
    return EF_OK;
}

ef_status ef_mpnn_refresh(int n, const float* p, void* pb, float* pf, cudaStream_t s) {
    refresh_kernel<<<nbm(n, 256), 256, 0, ef::counted(s)>>>(n, p, (__nv_bfloat16*)pb, pf);
    EF_CUDA(cudaGetLastError());
    return EF_OK;
}

ef_status ef_mpnn_alpha_combine(int64_t n, const float* Mv, const float* N, const double* dots, const uint8_t* mask,
                                float* z, cudaStream_t s) {
    alpha_combine_kernel<<<nbm(n, 256), 256, 0, ef::counted(s)>>>(n, Mv, N, dots, mask, z);
    EF_CUDA(cudaGetLastError());
    return EF_OK;
}
