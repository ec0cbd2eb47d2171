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

// ---- dense layer on the 5th-generation tensor cores ----------------------------------------------
// One CTA (4 warps) per tile of 128 nodes: X = [h | agg] (128 x 128) and W = [Ws | Wn] (64 x 128)
// are converted to BF16 into shared memory in the no-swizzle K-major layout of 8 x 16-byte core
// matrices, one thread issues 8 tcgen05.mma (M = 128, N = 64, K = 16, FP32 accumulate) into a
// 64-column TMEM accumulator, completion is signalled through an mbarrier (bounded wait), and
// each warp reads its 32 accumulator rows with tcgen05.ld for the epilogue q = relu(D),
// hout = h + q (h in FP32).
constexpr int TC_M = 128;                      // nodes per tile
constexpr int TC_K = 2 * H;                    // [h | agg]
constexpr int TC_A_BYTES = TC_M * TC_K * 2;    // 32 KB
constexpr int TC_B_BYTES = H * TC_K * 2;       // 16 KB
constexpr int TC_SMEM = TC_A_BYTES + TC_B_BYTES + 64;
constexpr long long TC_WAIT_LIMIT = 1ll << 22;       // mbarrier polls before giving up
constexpr long long TC_CLOCK_LIMIT = 2000000000ll;   // SM clocks before giving up (about 1 s)

// byte offset of element (row r, column k) in a no-swizzle K-major tile of K = 128 columns:
// core matrix (r / 8, k / 8) of 128 bytes, rows of 16 bytes inside
__device__ __forceinline__ uint32_t tc_offset(int r, int k) {
    return (uint32_t)((((r >> 3) * (TC_K / 8) + (k >> 3)) << 7) + ((r & 7) << 4) + ((k & 7) << 1));
}

// shared-memory matrix descriptor: start address, leading (K) and stride (8-row) byte offsets,
// descriptor version 1, no swizzle
__device__ __forceinline__ uint64_t tc_desc(uint32_t saddr, uint32_t lbo, uint32_t sbo) {
    uint64_t d = 0;
    d |= (uint64_t)((saddr & 0x3FFFF) >> 4);
    d |= (uint64_t)((lbo >> 4) & 0x3FFF) << 16;
    d |= (uint64_t)((sbo >> 4) & 0x3FFF) << 32;
    d |= (uint64_t)1 << 46;
    return d;
}

__global__ void __launch_bounds__(128) dense_tc_kernel(int nN, const float* __restrict__ h,
                                                       const float* __restrict__ agg, const float* __restrict__ Wl,
                                                       float* __restrict__ q, float* __restrict__ hout,
                                                       int* __restrict__ flags) {
    extern __shared__ __align__(1024) unsigned char tsm[];
    unsigned char* sA = tsm;
    unsigned char* sB = tsm + TC_A_BYTES;
    uint64_t* mbar = reinterpret_cast<uint64_t*>(tsm + TC_A_BYTES + TC_B_BYTES);
    uint32_t* tslot = reinterpret_cast<uint32_t*>(tsm + TC_A_BYTES + TC_B_BYTES + 16);
    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    const int m0 = blockIdx.x * TC_M;
    // operands -> BF16 in the core-matrix layout, one 16-byte core-matrix row (8 values) per step
    for (int i = tid; i < TC_M * (TC_K / 8); i += 128) {
        const int r = i / (TC_K / 8), k8 = i % (TC_K / 8);
        const int m = m0 + r;
        float4 v0 = make_float4(0.f, 0.f, 0.f, 0.f), v1 = v0;
        if (m < nN) {
            const float* src = k8 < H / 8 ? h + (int64_t)m * H + 8 * k8 : agg + (int64_t)m * H + 8 * (k8 - H / 8);
            v0 = *reinterpret_cast<const float4*>(src);
            v1 = *reinterpret_cast<const float4*>(src + 4);
        }
        __nv_bfloat162 b[4] = {__floats2bfloat162_rn(v0.x, v0.y), __floats2bfloat162_rn(v0.z, v0.w),
                               __floats2bfloat162_rn(v1.x, v1.y), __floats2bfloat162_rn(v1.z, v1.w)};
        *reinterpret_cast<uint4*>(sA + tc_offset(r, 8 * k8)) = *reinterpret_cast<uint4*>(b);
    }
    for (int i = tid; i < H * (TC_K / 8); i += 128) {
        const int c = i / (TC_K / 8), k8 = i % (TC_K / 8);
        const float* src = k8 < H / 8 ? Wl + c * H + 8 * k8 : Wl + H * H + c * H + 8 * (k8 - H / 8);
        const float4 v0 = *reinterpret_cast<const float4*>(src);
        const float4 v1 = *reinterpret_cast<const float4*>(src + 4);
        __nv_bfloat162 b[4] = {__floats2bfloat162_rn(v0.x, v0.y), __floats2bfloat162_rn(v0.z, v0.w),
                               __floats2bfloat162_rn(v1.x, v1.y), __floats2bfloat162_rn(v1.z, v1.w)};
        *reinterpret_cast<uint4*>(sB + tc_offset(c, 8 * k8)) = *reinterpret_cast<uint4*>(b);
    }
    const uint32_t mbarAddr = (uint32_t)__cvta_generic_to_shared(mbar);
    if (tid == 0) {
        asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(mbarAddr));
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    if (warp == 0) {
        const uint32_t slotAddr = (uint32_t)__cvta_generic_to_shared(tslot);
        asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], 64;" ::"r"(slotAddr));
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;");
        asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
    }
    asm volatile("fence.proxy.async.shared::cta;" ::: "memory");  // generic stores -> async proxy
    __syncthreads();
    asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
    const uint32_t tmem = *tslot;
    if (tid == 0) {
        const uint32_t aBase = (uint32_t)__cvta_generic_to_shared(sA);
        const uint32_t bBase = (uint32_t)__cvta_generic_to_shared(sB);
        const uint32_t idesc = (1u << 4) | (1u << 7) | (1u << 10) | ((uint32_t)(H >> 3) << 17) |
                               ((uint32_t)(TC_M >> 4) << 24);  // F32 accum, BF16 A/B, K-major, N = 64, M = 128
#pragma unroll
        for (int ks = 0; ks < TC_K / 16; ++ks) {
            const uint64_t ad = tc_desc(aBase + ks * 256, 128, (TC_K / 8) * 128);
            const uint64_t bd = tc_desc(bBase + ks * 256, 128, (TC_K / 8) * 128);
            const uint32_t acc = ks > 0 ? 1u : 0u;
            asm volatile(
                "{\n.reg .pred p;\nsetp.ne.b32 p, %4, 0;\n"
                "tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n}" ::"r"(tmem),
                "l"(ad), "l"(bd), "r"(idesc), "r"(acc));
        }
        asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(mbarAddr)
                     : "memory");
    }
    // bounded wait for the accumulator (phase 0): a poll count and a clock limit of about a second
    long long polls = 0;
    const long long t0 = clock64();
    uint32_t done = 0;
    while (!done) {
        asm volatile(
            "{\n.reg .pred p;\nmbarrier.try_wait.parity.shared::cta.b64 p, [%1], 0;\nselp.u32 %0, 1, 0, p;\n}"
            : "=r"(done)
            : "r"(mbarAddr)
            : "memory");
        if (!done && (++polls > TC_WAIT_LIMIT || clock64() - t0 > TC_CLOCK_LIMIT)) break;
    }
    done = __syncthreads_and(done);  // the whole CTA reads the accumulator, or none of it
    asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
    if (done) {
        // warp w owns accumulator rows (TMEM lanes) 32w .. 32w + 31; 64 FP32 columns each
        uint32_t r[64];
        const uint32_t taddr = tmem + ((uint32_t)(warp * 32) << 16);
        asm volatile(
            "tcgen05.ld.sync.aligned.32x32b.x64.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15,"
            "%16,%17,%18,%19,%20,%21,%22,%23,%24,%25,%26,%27,%28,%29,%30,%31,%32,%33,%34,%35,%36,%37,%38,%39,"
            "%40,%41,%42,%43,%44,%45,%46,%47,%48,%49,%50,%51,%52,%53,%54,%55,%56,%57,%58,%59,%60,%61,%62,%63}, "
            "[%64];"
            : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]),
              "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15]),
              "=r"(r[16]), "=r"(r[17]), "=r"(r[18]), "=r"(r[19]), "=r"(r[20]), "=r"(r[21]), "=r"(r[22]),
              "=r"(r[23]), "=r"(r[24]), "=r"(r[25]), "=r"(r[26]), "=r"(r[27]), "=r"(r[28]), "=r"(r[29]),
              "=r"(r[30]), "=r"(r[31]), "=r"(r[32]), "=r"(r[33]), "=r"(r[34]), "=r"(r[35]), "=r"(r[36]),
              "=r"(r[37]), "=r"(r[38]), "=r"(r[39]), "=r"(r[40]), "=r"(r[41]), "=r"(r[42]), "=r"(r[43]),
              "=r"(r[44]), "=r"(r[45]), "=r"(r[46]), "=r"(r[47]), "=r"(r[48]), "=r"(r[49]), "=r"(r[50]),
              "=r"(r[51]), "=r"(r[52]), "=r"(r[53]), "=r"(r[54]), "=r"(r[55]), "=r"(r[56]), "=r"(r[57]),
              "=r"(r[58]), "=r"(r[59]), "=r"(r[60]), "=r"(r[61]), "=r"(r[62]), "=r"(r[63])
            : "r"(taddr));
        asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
        // stage relu(D) row by row through shared memory (the operand tiles are no longer read once
        // the MMAs completed; 128 x 65 words), padded by one word per row against bank conflicts,
        // then write q and hout coalesced
        float* sD = reinterpret_cast<float*>(sA);
        const int row = warp * 32 + lane;
#pragma unroll
        for (int c = 0; c < H; ++c) sD[row * (H + 1) + c] = fmaxf(__uint_as_float(r[c]), 0.f);
    }
    asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
    __syncthreads();
    if (done) {
        const float* sD = reinterpret_cast<const float*>(sA);
        for (int i = tid; i < TC_M * H; i += 128) {
            const int rr = i / H, c = i % H;
            const int m = m0 + rr;
            if (m >= nN) continue;
            const float qq = sD[rr * (H + 1) + c];
            q[(int64_t)m * H + c] = qq;
            hout[(int64_t)m * H + c] = h[(int64_t)m * H + c] + qq;
        }
    } else if (tid == 0) {
        // the accumulator never became ready: this tile's output is skipped, and an MMA still in
        // flight may write TMEM columns after the dealloc below, so the host must discard the
        // whole network pass and stop using the tensor-core layer (see EF_FLAG_TCWAIT)
        atomicOr(flags, EF_FLAG_TCWAIT);
    }
    if (warp == 0) asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, 64;" ::"r"(tmem));
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
    // per-thread and per-warp sums in FP32 (a thread holds a few elements), the CTA's warp sums
    // and the sum over CTAs in FP64: FP64 is a narrow pipe on this GPU
    __shared__ float red[8][3];
    float acc[3] = {0.f, 0.f, 0.f};
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
        if (groups == 0) {
            if (mask && mask[i]) continue;
            acc[0] = fmaf(z[i], e[i], acc[0]);
        } else if (groups == 3) {
            const int g = (int)((i % FIN) / 3);
            const float v = z[i];
            acc[0] += g == 0 ? v * v : 0.f;
            acc[1] += g == 1 ? v * v : 0.f;
            acc[2] += g == 2 ? v * v : 0.f;
        } else {
            if (mask && mask[i]) continue;
            const float d = z[i] - (e ? e[i] : 0.f);
            acc[0] = fmaf(d, d, acc[0]);
        }
    }
    const int lane = threadIdx.x & 31, wp = threadIdx.x >> 5;
#pragma unroll
    for (int g = 0; g < 3; ++g) {
        float a = acc[g];
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) a += __shfl_xor_sync(0xffffffffu, a, o);
        if (lane == 0) red[wp][g] = a;
    }
    __syncthreads();
    if (threadIdx.x < 3) {
        double t = 0.0;
        for (int w = 0; w < (int)(blockDim.x >> 5); ++w) t += (double)red[w][threadIdx.x];
        part[(int64_t)blockIdx.x * 3 + threadIdx.x] = t;
    }
}

// out[g] = sum_c part[c][g], one warp per g: lane-strided sums, then a fixed shuffle tree
// (fac: optional, 1 / sqrt(out[0]) in FP32, 1 when out[0] is not positive -- the power
// iteration's normalisation factor, formed once instead of per element)
__global__ void sumsq_final_kernel(int nPart, const double* __restrict__ part, double* __restrict__ out,
                                   float* __restrict__ fac) {
    const int g = threadIdx.x >> 5, lane = threadIdx.x & 31;
    if (g >= 3) return;
    double t = 0.0;
    for (int c = lane; c < nPart; c += 32) t += part[(int64_t)c * 3 + g];
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) t += __shfl_xor_sync(0xffffffffu, t, o);
    if (lane == 0) {
        out[g] = t;
        if (g == 0 && fac) *fac = t > 0.0 ? (float)(1.0 / sqrt(t)) : 1.f;
    }
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
    EF_CUDA(cudaFuncSetAttribute(dense_tc_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, TC_SMEM));
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
ef_status ef_mpnn_dense(int tc, int nN, const float* h, const float* agg, const float* Wl, float* q, float* hout,
                        int* flags, cudaStream_t s);

// tc != 0: dense layers on the tensor cores (flags receives a tile's timeout), else FP32 CUDA cores
ef_status ef_mpnn_forward(int nN, const int32_t* rowPtr, const int32_t* colIdx, const float* a, const float* P,
                          const float* f, const float* base, const uint8_t* mask, float so, float* acts, float* z,
                          int tc, int* flags, cudaStream_t s) {
    const int64_t NH = (int64_t)nN * H;
    float* h0 = acts;
    input_kernel<<<nbm(NH, 256), 256, 0, ef::counted(s)>>>(nN, f, P, h0);
    const float* hprev = h0;
    for (int l = 0; l < NL; ++l) {
        float* q = acts + NH * (1 + 3 * l);
        float* hl = q + NH;
        float* agg = hl + NH;
        aggregate_kernel<<<nbm((int64_t)nN * 32, 256), 256, 0, ef::counted(s)>>>(nN, rowPtr, colIdx, a, hprev, agg, 0);
        const ef_status st = ef_mpnn_dense(tc, nN, hprev, agg, P + OFF_L0 + l * PER_LAYER, q, hl, flags, s);
        if (st != EF_OK) return st;
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
                        int nPart, double* out, cudaStream_t s, float* fac) {
    sumsq_partial_kernel<<<nPart, 256, 0, ef::counted(s)>>>(n, groups, z, e, mask, part);
    sumsq_final_kernel<<<1, 96, 0, ef::counted(s)>>>(nPart, part, out, fac);
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

// one dense layer, q = relu(Ws h + Wn agg), hout = h + q, on the tensor cores (tc != 0) or the
// FP32 CUDA cores; flags receives EF_FLAG_TCWAIT if a tensor-core tile gave up waiting
ef_status ef_mpnn_dense(int tc, int nN, const float* h, const float* agg, const float* Wl, float* q, float* hout,
                        int* flags, cudaStream_t s) {
    if (nN == 0) return EF_OK;
    if (tc)
        dense_tc_kernel<<<nbm(nN, TC_M), 128, TC_SMEM, ef::counted(s)>>>(nN, h, agg, Wl, q, hout, flags);
    else
        dense_kernel<<<nbm(nN, TILE), 256, kDenseSmem, ef::counted(s)>>>(nN, h, agg, Wl, q, hout);
    EF_CUDA(cudaGetLastError());
    return EF_OK;
}

// host-array check entry: one dense layer on the tensor cores (tc = 1) or the CUDA cores (tc = 0)
ef_status ef_mpnn_dense_eval_host(int tc, int nN, const float* h, const float* agg, const float* W, float* q,
                                  float* hout, int* flagsOut, cudaStream_t s) {
    const ef_status su = ef_mpnn_setup_kernels();
    if (su != EF_OK) return su;
    const size_t nh = (size_t)nN * H;
    float *dh = nullptr, *da = nullptr, *dw = nullptr, *dq = nullptr, *dho = nullptr;
    int* df = nullptr;
    auto fin = [&](ef_status r) {
        cudaFree(dh);
        cudaFree(da);
        cudaFree(dw);
        cudaFree(dq);
        cudaFree(dho);
        cudaFree(df);
        return r;
    };
    if (cudaMalloc(&dh, nh * 4) != cudaSuccess || cudaMalloc(&da, nh * 4) != cudaSuccess ||
        cudaMalloc(&dw, 2 * H * H * 4) != cudaSuccess || cudaMalloc(&dq, nh * 4) != cudaSuccess ||
        cudaMalloc(&dho, nh * 4) != cudaSuccess || cudaMalloc(&df, 4) != cudaSuccess) {
        ef_set_error("ef_mpnn_dense_eval: cudaMalloc failed");
        return fin(EF_ERR_CUDA);
    }
    if (cudaMemcpyAsync(dh, h, nh * 4, cudaMemcpyHostToDevice, s) != cudaSuccess ||
        cudaMemcpyAsync(da, agg, nh * 4, cudaMemcpyHostToDevice, s) != cudaSuccess ||
        cudaMemcpyAsync(dw, W, 2 * H * H * 4, cudaMemcpyHostToDevice, s) != cudaSuccess ||
        cudaMemsetAsync(df, 0, 4, s) != cudaSuccess)
        return fin(EF_ERR_CUDA);
    const ef_status st = ef_mpnn_dense(tc, nN, dh, da, dw, dq, dho, df, s);
    if (st != EF_OK) return fin(st);
    if (cudaMemcpyAsync(q, dq, nh * 4, cudaMemcpyDeviceToHost, s) != cudaSuccess ||
        cudaMemcpyAsync(hout, dho, nh * 4, cudaMemcpyDeviceToHost, s) != cudaSuccess ||
        cudaMemcpyAsync(flagsOut, df, 4, cudaMemcpyDeviceToHost, s) != cudaSuccess ||
        cudaStreamSynchronize(s) != cudaSuccess) {
        ef_set_error("ef_mpnn_dense_eval: copy back failed");
        return fin(EF_ERR_CUDA);
    }
    return fin(EF_OK);
}
