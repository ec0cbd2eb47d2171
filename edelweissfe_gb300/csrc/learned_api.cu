// C ABI of the learned FGMRES correction: network state, training pairs (from the solves or
// given), GPU training with the forward, backward and Adam kernels of mpnn.cu, and the
// verification entry points on host arrays.

#include <random>

#include "ctx.h"

static void nn_normal(std::mt19937_64& g, float sd, float* out, int n) {
    const double two_pi = 6.283185307179586;
    for (int i = 0; i < n; i += 2) {
        const double u1 = ((g() >> 11) + 1.0) * (1.0 / 9007199254740993.0);
        const double u2 = (g() >> 11) * (1.0 / 9007199254740992.0);
        const double rad = sqrt(-2.0 * log(u1));
        out[i] = (float)(sd * rad * cos(two_pi * u2));
        if (i + 1 < n) out[i + 1] = (float)(sd * rad * sin(two_pi * u2));
    }
}

// block (m, n) -> position of block (n, m) in the (structurally symmetric) block pattern
static ef_status nn_transpose_map(const std::vector<int32_t>& rowPtr, const std::vector<int32_t>& colIdx,
                                  std::vector<int64_t>& tpos) {
    const int64_t nN = (int64_t)rowPtr.size() - 1;
    tpos.assign(colIdx.size(), -1);
    for (int64_t m = 0; m < nN; ++m)
        for (int32_t k = rowPtr[m]; k < rowPtr[m + 1]; ++k) {
            const int32_t n = colIdx[k];
            const auto b = colIdx.begin() + rowPtr[n], e = colIdx.begin() + rowPtr[n + 1];
            const auto it = std::lower_bound(b, e, (int32_t)m);
            if (it == e || *it != (int32_t)m) {
                ef_set_error("learned correction: block pattern is not structurally symmetric");
                return EF_ERR_STATE;
            }
            tpos[k] = it - colIdx.begin();
        }
    return EF_OK;
}

static ef_status nn_upload_params(ef_ctx* c, const float* hp, cudaStream_t s) {
    const int np = ef_mpnn_nparam();
    EF_CUDA(cudaMemcpyAsync(c->nnP, hp, sizeof(float) * np, cudaMemcpyHostToDevice, s));
    EF_CUDA(cudaMemsetAsync(c->nnM1, 0, sizeof(float) * np, s));
    EF_CUDA(cudaMemsetAsync(c->nnM2, 0, sizeof(float) * np, s));
    EF_CHECK(ef_mpnn_refresh(np, c->nnP, c->nnPb, c->nnPf, s));
    EF_CUDA(cudaStreamSynchronize(s));
    c->nnStep = 0;
    return EF_OK;
}

// the stored copy of the current system (K values and edge weights), evicting the oldest one
// (and the pairs taken from it) when the store is full
ef_status nn_current_system(ef_ctx* c, cudaStream_t s, int* out) {
    for (size_t i = 0; i < c->nnSystems.size(); ++i)
        if (c->nnSystems[i].version == c->nnVersion) {
            *out = (int)i;
            return EF_OK;
        }
    int slot = -1;
    std::vector<int> used(c->nnSystems.size(), 0);
    for (const auto& S : c->nnSamples)
        if (S.sys >= 0) used[S.sys] = 1;
    for (size_t i = 0; i < c->nnSystems.size() && slot < 0; ++i)
        if (!used[i]) slot = (int)i;
    if (slot < 0 && (int)c->nnSystems.size() < c->nnMaxSystems) {
        ef_status st = EF_OK;
        ef_ctx::NNSystem Y;
        Y.K = dalloc<float>((size_t)c->nBlocks * 9, &st);
        Y.a = dalloc<float>(c->nBlocks, &st);
        c->nnSystems.push_back(Y);
        if (st != EF_OK) return st;
        slot = (int)c->nnSystems.size() - 1;
    }
    if (slot < 0) {  // evict the oldest system
        slot = 0;
        for (size_t i = 1; i < c->nnSystems.size(); ++i)
            if (c->nnSystems[i].version < c->nnSystems[slot].version) slot = (int)i;
        for (auto& S : c->nnSamples)
            if (S.sys == slot) S.sys = -1;
    }
    ef_ctx::NNSystem& Y = c->nnSystems[slot];
    EF_CHECK(nn_edge_refresh(c, s, true));
    EF_CUDA(cudaMemcpyAsync(Y.K, c->dBsrVals, sizeof(float) * 9 * c->nBlocks, cudaMemcpyDeviceToDevice, s));
    EF_CUDA(cudaMemcpyAsync(Y.a, c->nnA, sizeof(float) * c->nBlocks, cudaMemcpyDeviceToDevice, s));
    Y.version = c->nnVersion;
    *out = slot;
    return EF_OK;
}

// adds the training pair (r, e) with K e = r (free DOFs, FP32 device vectors; e may be null:
// an input without its correction), scaled to rms(e) = 1 (rms(r) = 1 without e); the multigrid
// hierarchy and edge weights must be current.  Features: [Mv, rho, D^-1 rho], rho = r - K Mv.
ef_status nn_add_sample(ef_ctx* c, const float* r, const float* e, cudaStream_t s) {
    const int64_t n = c->nDof;
    const int64_t nN = c->nNodes;
    if (c->nnMaxSamples == 0) return EF_OK;
    double* out = c->nnRed + 3 * c->nnPartN;
    double h[3] = {0, 0, 0};
    if (e) {
        EF_CHECK(ef_mpnn_sumsq(n, 1, e, nullptr, c->dMask, c->nnRed, c->nnPartN, out, s));
        EF_CUDA(cudaMemcpyAsync(&h[0], out, sizeof(double), cudaMemcpyDeviceToHost, s));
        EF_CHECK(ef_mpnn_sumsq(n, 0, e, r, c->dMask, c->nnRed, c->nnPartN, out + 3, s));
        EF_CUDA(cudaMemcpyAsync(&h[1], out + 3, sizeof(double), cudaMemcpyDeviceToHost, s));
    }
    EF_CHECK(ef_mpnn_sumsq(n, 1, r, nullptr, c->dMask, c->nnRed, c->nnPartN, out, s));
    EF_CUDA(cudaMemcpyAsync(&h[2], out, sizeof(double), cudaMemcpyDeviceToHost, s));
    EF_CUDA(cudaStreamSynchronize(s));
    const double ss = e ? h[0] : h[2];
    if (!(ss > 0.0) || !(ss < 1e300) || !(h[2] > 0.0) || (e && !(h[1] > 0.0))) return EF_OK;  // nothing to learn
    int sys = -1;
    EF_CHECK(nn_current_system(c, s, &sys));
    size_t slot = c->nnSamples.size();
    for (size_t i = 0; i < c->nnSamples.size(); ++i)
        if (c->nnSamples[i].sys < 0) {
            slot = i;
            break;
        }
    if (slot == c->nnSamples.size()) {
        if ((int)c->nnSamples.size() < c->nnMaxSamples) {
            ef_status st = EF_OK;
            ef_ctx::NNSample S;
            S.f = dalloc<float>(9 * nN, &st);
            S.base = dalloc<float>(n, &st);
            S.r = dalloc<float>(n, &st);
            S.e = dalloc<float>(n, &st);
            c->nnSamples.push_back(S);
            if (st != EF_OK) return st;
        } else {
            slot = (size_t)(c->nnAdded % c->nnMaxSamples);
        }
    }
    c->nnAdded++;
    ef_ctx::NNSample& S = c->nnSamples[slot];
    const double inv2 = (double)n / ss;
    S.sys = sys;
    S.hasE = e != nullptr;
    S.ee = h[0] * inv2;
    S.er = h[1] * inv2;
    S.rr = h[2] * inv2;
    const float inv = (float)sqrt(inv2);
    EF_CUDA(cudaMemcpyAsync(c->vcIn, r, sizeof(float) * n, cudaMemcpyDeviceToDevice, s));
    c->vcInStale = true;
    EF_CHECK(apply_base(c, s));
    EF_CHECK(ef_launch_spmv_f32((int)nN, c->dRowPtr, c->dColIdx, (const float*)c->dBsrVals, c->vcOut, c->dMask,
                                c->nnKd, s));
    EF_CHECK(ef_launch_sub(n, c->vcIn, c->nnKd, c->nnRho, s));
    EF_CHECK(ef_launch_features((int)nN, c->vcOut, c->nnRho, (const float*)c->dBinv, 1.f, 1.f, 1.f, S.f, s));
    EF_CUDA(cudaMemcpyAsync(S.base, c->vcOut, sizeof(float) * n, cudaMemcpyDeviceToDevice, s));
    EF_CUDA(cudaMemcpyAsync(S.r, c->vcIn, sizeof(float) * n, cudaMemcpyDeviceToDevice, s));
    if (e) EF_CUDA(cudaMemcpyAsync(S.e, e, sizeof(float) * n, cudaMemcpyDeviceToDevice, s));
    EF_CHECK(ef_mpnn_scale(9 * nN, S.f, inv, s));
    EF_CHECK(ef_mpnn_scale(n, S.base, inv, s));
    EF_CHECK(ef_mpnn_scale(n, S.r, inv, s));
    if (e) EF_CHECK(ef_mpnn_scale(n, S.e, inv, s));
    return EF_OK;
}

// pairs from the iterates of a converged FGMRES solve: e_k = x - x_k, r_k = K e_k
ef_status nn_collect_snapshots(ef_ctx* c, const float* x, cudaStream_t s) {
    const int64_t n = c->nDof;
    for (int k = 0; k < c->nnSnapCount; ++k) {
        float* ek = c->nnSnaps[k];
        EF_CHECK(ef_launch_sub(n, x, ek, ek, s));
        EF_CHECK(ef_launch_spmv_f32((int)c->nNodes, c->dRowPtr, c->dColIdx, (const float*)c->dBsrVals, ek, c->dMask,
                                    c->fgW, s));
        EF_CHECK(nn_add_sample(c, c->fgW, ek, s));
    }
    c->nnSnapCount = 0;
    return EF_OK;
}

ef_status nn_snapshot_buffer(ef_ctx* c, float** out) {
    if (c->nnSnapCount >= (int)c->nnSnaps.size()) {
        ef_status st = EF_OK;
        float* p = dalloc<float>(c->nDof, &st);
        if (!p) return st;
        c->nnSnaps.push_back(p);
    }
    *out = c->nnSnaps[c->nnSnapCount++];
    return EF_OK;
}

// epochs of Adam over the stored pairs (shuffled deterministically); epochs = 0 only evaluates.
// Loss of a pair with d = z - e, relative to the same norm of e:
//   norm 0: |d|^2 / |e|^2,  norm 1: d.K d / e.K e,  norm 2: |K d|^2 / |K e|^2
// (K the system the pair was taken from); the mean over the pairs is reported.
static ef_status nn_train(ef_ctx* c, int epochs, float lr, int norm, double* lossFirst, double* lossLast,
                          cudaStream_t s) {
    std::vector<int> valid;
    for (size_t i = 0; i < c->nnSamples.size(); ++i)
        if (c->nnSamples[i].sys >= 0 && (norm == 2 || c->nnSamples[i].hasE)) valid.push_back((int)i);
    const int nS = (int)valid.size();
    if (nS == 0) {
        ef_set_error("ef_mpnn_train: no training pairs");
        return EF_ERR_STATE;
    }
    const int64_t n = c->nDof, nN = c->nNodes;
    double* out = c->nnRed + 3 * c->nnPartN;
    if (!c->nnScalesSet) {
        // feature group scales: 1 / rms of each group over the stored pairs
        double acc[3] = {0, 0, 0};
        for (int i : valid) {
            EF_CHECK(ef_mpnn_sumsq(9 * nN, 3, c->nnSamples[i].f, nullptr, nullptr, c->nnRed, c->nnPartN, out, s));
            double h[3];
            EF_CUDA(cudaMemcpyAsync(h, out, sizeof(h), cudaMemcpyDeviceToHost, s));
            EF_CUDA(cudaStreamSynchronize(s));
            for (int g = 0; g < 3; ++g) acc[g] += h[g];
        }
        for (int g = 0; g < 3; ++g) {
            const double rms = sqrt(acc[g] / (3.0 * nN * nS));
            c->nnS[g] = rms > 0.0 ? (float)(1.0 / rms) : 1.f;
        }
        c->nnScalesSet = true;
        if (c->nnGraph) {
            cudaGraphExecDestroy(c->nnGraph);
            c->nnGraph = nullptr;
        }
    }
    ef_status st = EF_OK;
    double* lossBuf = dalloc<double>(3 * (size_t)nS, &st);
    if (!lossBuf) return st;
    std::vector<double> hl(3 * (size_t)nS);
    std::vector<int> order(nS);
    const int np = ef_mpnn_nparam();
    for (int ep = 0; ep < std::max(epochs, 1); ++ep) {
        for (int i = 0; i < nS; ++i) order[i] = i;
        std::mt19937_64 g(0x5eed0000ull + (uint64_t)c->nnStep + (uint64_t)ep);
        for (int i = nS - 1; i > 0; --i) std::swap(order[i], order[(int)(g() % (uint64_t)(i + 1))]);
        for (int t = 0; t < nS; ++t) {
            const ef_ctx::NNSample& S = c->nnSamples[valid[order[t]]];
            const ef_ctx::NNSystem& Y = c->nnSystems[S.sys];
            EF_CHECK(ef_mpnn_scale_features((int)nN, S.f, c->nnS[0], c->nnS[1], c->nnS[2], c->nnF, s));
            EF_CHECK(ef_mpnn_forward((int)nN, c->dRowPtr, c->dColIdx, Y.a, c->nnPf, c->nnF, S.base, c->dMask, c->nnSo,
                                     c->nnActs, c->vcOut2, c->nnTensorCores, c->dFlags, s));
            // rho = dL/dz up to the factor scale: d, K d or K (K z - r), d = z - e
            const float* rho = c->nnD;
            double ref = S.ee;
            double* lb = lossBuf + 3 * order[t];
            if (norm == 0) {
                EF_CHECK(ef_launch_sub(n, c->vcOut2, S.e, c->nnD, s));
                EF_CHECK(ef_mpnn_sumsq(n, 1, c->nnD, nullptr, c->dMask, c->nnRed, c->nnPartN, lb, s));
            } else if (norm == 1) {
                EF_CHECK(ef_launch_sub(n, c->vcOut2, S.e, c->nnD, s));
                EF_CHECK(ef_launch_spmv_f32((int)nN, c->dRowPtr, c->dColIdx, Y.K, c->nnD, c->dMask, c->nnKd, s));
                EF_CHECK(ef_mpnn_sumsq(n, 0, c->nnD, c->nnKd, c->dMask, c->nnRed, c->nnPartN, lb, s));
                rho = c->nnKd;
                ref = S.er;
            } else {
                EF_CHECK(ef_launch_spmv_f32((int)nN, c->dRowPtr, c->dColIdx, Y.K, c->vcOut2, c->dMask, c->nnKd, s));
                EF_CHECK(ef_launch_sub(n, c->nnKd, S.r, c->nnKd, s));
                EF_CHECK(ef_mpnn_sumsq(n, 1, c->nnKd, nullptr, c->dMask, c->nnRed, c->nnPartN, lb, s));
                EF_CHECK(ef_launch_spmv_f32((int)nN, c->dRowPtr, c->dColIdx, Y.K, c->nnKd, c->dMask, c->nnD, s));
                rho = c->nnD;
                ref = S.rr;
            }
            if (epochs == 0) continue;
            // gradient of 0.5 * |.|^2 / ref: backward with z := rho, e := 0, scale 1 / ref
            EF_CHECK(ef_launch_gather_f32(c->nBlocks, c->nnTpos, Y.a, c->nnAT, s));
            EF_CHECK(ef_mpnn_backward((int)nN, c->dRowPtr, c->dColIdx, c->nnAT, c->nnPf, c->nnF, c->nnActs, rho,
                                      nullptr, c->dMask, (float)(1.0 / ref), c->nnSo, c->nnG, c->nnWork, c->nnPart,
                                      c->nnPartN, s));
            EF_CHECK(ef_mpnn_adam(np, c->nnP, c->nnG, c->nnM1, c->nnM2, lr, 0.9f, 0.999f, 1e-8f, ++c->nnStep, c->nnPb,
                                  c->nnPf, s));
        }
        EF_CUDA(cudaMemcpyAsync(hl.data(), lossBuf, sizeof(double) * hl.size(), cudaMemcpyDeviceToHost, s));
        EF_CUDA(cudaStreamSynchronize(s));
        double mean = 0.0;
        for (int t = 0; t < nS; ++t) {
            const ef_ctx::NNSample& S = c->nnSamples[valid[t]];
            mean += hl[3 * t] / (norm == 0 ? S.ee : (norm == 1 ? S.er : S.rr));
        }
        mean /= nS;
        if (ep == 0 && lossFirst) *lossFirst = mean;
        if (lossLast) *lossLast = mean;
    }
    cudaFree(lossBuf);
    return EF_OK;
}

// FGMRES(m) on the free DOFs for K x = b (FP32 vectors, FP64 reductions and Hessenberg);
// x starts at 0; stops at ||b - K x|| <= rtol ||b|| (Arnoldi estimate) or maxIter
ef_status ef_mpnn_dense_eval(int tensorCores, int nNodes, const float* h, const float* agg, const float* W,
                             float* q, float* hout, int* flags, void* stream) {
    if (nNodes <= 0 || !h || !agg || !W || !q || !hout || !flags) return EF_ERR_ARG;
    return ef_mpnn_dense_eval_host(tensorCores ? 1 : 0, nNodes, h, agg, W, q, hout, flags, (cudaStream_t)stream);
}

int64_t ef_kernel_launches(void) { return (int64_t)ef::launches(); }

int ef_mpnn_param_count(void) { return ef_mpnn_nparam(); }

ef_status ef_mpnn_init(ef_ctx* c, uint64_t seed, int maxSamples) {
    EF_REQUIRE_FINALIZED(c);
    if (maxSamples < 0) return EF_ERR_ARG;
    if (c->keFp64) {
        ef_set_error("ef_mpnn_init: the learned correction runs inside the FP32 FGMRES (mixed mode)");
        return EF_ERR_ARG;
    }
    EF_CHECK(ef_mpnn_setup_kernels());
    const int np = ef_mpnn_nparam(), H = ef_mpnn_hidden();
    if (!c->nnInit) {
        ef_status st = EF_OK;
        const int64_t nN = c->nNodes, NH = nN * H;
        c->nnP = dalloc<float>(np, &st);
        c->nnPf = dalloc<float>(np, &st);
        c->nnM1 = dalloc<float>(np, &st);
        c->nnM2 = dalloc<float>(np, &st);
        c->nnG = dalloc<float>(np, &st);
        c->nnPb = dalloc<uint16_t>(np, &st);
        c->nnActs = dalloc<float>(10 * NH, &st);
        c->nnF = dalloc<float>(9 * nN, &st);
        c->nnWork = dalloc<float>(4 * NH, &st);
        c->nnPartN = 2 * c->nSM;
        c->nnPart = dalloc<float>((size_t)c->nnPartN * H * H, &st);
        c->nnA = dalloc<float>(c->nBlocks, &st);
        c->nnAT = dalloc<float>(c->nBlocks, &st);
        c->nnTpos = dalloc<int64_t>(c->nBlocks, &st);
        if (!c->nnRed) c->nnRed = dalloc<double>(3 * (size_t)c->nnPartN + 8, &st);
        c->vcOut2 = dalloc<float>(c->nDof, &st);
        c->nnD = dalloc<float>(c->nDof, &st);
        c->nnKd = dalloc<float>(c->nDof, &st);
        c->nnRho = dalloc<float>(c->nDof, &st);
        c->nnN = dalloc<float>(c->nDof, &st);
        c->nnKN = dalloc<float>(c->nDof, &st);
        if (st != EF_OK) return st;
        std::vector<int64_t> tpos;
        EF_CHECK(nn_transpose_map(c->hRowPtr0, c->hColIdx0, tpos));
        EF_CUDA(cudaMemcpy(c->nnTpos, tpos.data(), sizeof(int64_t) * tpos.size(), cudaMemcpyHostToDevice));
        c->nnInit = true;
        c->amgStale = true;  // edge weights are computed with the next refresh
        c->nnEdgeStale = true;
    }
    // He-scaled normal weights; residual branches damped; output layer zero (z = Mv at start)
    std::mt19937_64 g(seed);
    std::vector<float> hp(np, 0.f);
    nn_normal(g, (float)sqrt(2.0 / 9.0), hp.data(), H * 9);
    for (int l = 0; l < 3; ++l) nn_normal(g, (float)(0.5 * sqrt(2.0 / (2.0 * H))), hp.data() + ef_mpnn_layer_offset(l), 2 * H * H);
    EF_CHECK(nn_upload_params(c, hp.data(), nullptr));
    c->nnScalesSet = false;
    c->nnS[0] = c->nnS[1] = c->nnS[2] = 1.f;
    c->nnSo = 1.f;
    c->nnMaxSamples = maxSamples;
    c->nnMaxSystems = std::min(maxSamples, 16);
    if (c->nnGraph) {
        cudaGraphExecDestroy(c->nnGraph);
        c->nnGraph = nullptr;
    }
    return EF_OK;
}

ef_status ef_mpnn_set_params(ef_ctx* c, const float* params, const float* scales) {
    EF_REQUIRE_FINALIZED(c);
    if (!c->nnInit) {
        ef_set_error("ef_mpnn_set_params: call ef_mpnn_init first");
        return EF_ERR_STATE;
    }
    if (params) EF_CHECK(nn_upload_params(c, params, nullptr));
    if (scales) {
        for (int i = 0; i < 3; ++i) c->nnS[i] = scales[i];
        c->nnSo = scales[3];
        c->nnScalesSet = true;
        if (c->nnGraph) {
            cudaGraphExecDestroy(c->nnGraph);
            c->nnGraph = nullptr;
        }
    }
    return EF_OK;
}

ef_status ef_mpnn_get_params(ef_ctx* c, float* params, float* scales) {
    EF_REQUIRE_FINALIZED(c);
    if (!c->nnInit) {
        ef_set_error("ef_mpnn_get_params: call ef_mpnn_init first");
        return EF_ERR_STATE;
    }
    if (params) EF_CUDA(cudaMemcpy(params, c->nnP, sizeof(float) * ef_mpnn_nparam(), cudaMemcpyDeviceToHost));
    if (scales) {
        for (int i = 0; i < 3; ++i) scales[i] = c->nnS[i];
        scales[3] = c->nnSo;
    }
    return EF_OK;
}

ef_status ef_mpnn_enable(ef_ctx* c, int on) {
    EF_REQUIRE_FINALIZED(c);
    if (on && !c->nnInit) {
        ef_set_error("ef_mpnn_enable: call ef_mpnn_init first");
        return EF_ERR_STATE;
    }
    c->nnOn = on != 0;
    return EF_OK;
}

ef_status ef_mpnn_collect(ef_ctx* c, int every, int maxPerSolve, int kind) {
    EF_REQUIRE_FINALIZED(c);
    if (every < 0 || maxPerSolve < 0 || kind < 0 || kind > 1) return EF_ERR_ARG;
    c->nnKind = kind;
    if ((every > 0 || maxPerSolve > 0) && !c->nnInit) {
        ef_set_error("ef_mpnn_collect: call ef_mpnn_init first");
        return EF_ERR_STATE;
    }
    c->nnEvery = every;
    c->nnMaxPerSolve = maxPerSolve;
    return EF_OK;
}

ef_status ef_mpnn_add_sample(ef_ctx* c, const double* r, const double* e, void* stream) {
    EF_REQUIRE_FINALIZED(c);
    if (!r || !e) return EF_ERR_ARG;
    if (!c->nnInit) {
        ef_set_error("ef_mpnn_add_sample: call ef_mpnn_init first");
        return EF_ERR_STATE;
    }
    if (c->nnMaxSamples == 0) return EF_OK;
    cudaStream_t s = (cudaStream_t)stream;
    if (c->fgPc == EF_FGMRES_PC_MULTIGRID) {
        EF_CHECK(amg_build(c));
        EF_CHECK(amg_refresh(c, s));
    } else {
        EF_CHECK(amg_workspace(c));
        EF_CHECK(nn_edge_refresh(c, s));
    }
    const int64_t n = c->nDof;
    float* rf = (float*)c->w32[5];
    float* ef = (float*)c->w32[6];
    EF_CHECK(ef_launch_masked_copy(n, r, c->dMask, 0, 1.0, rf, 0, s));
    EF_CHECK(ef_launch_masked_copy(n, e, c->dMask, 0, 1.0, ef, 0, s));
    return nn_add_sample(c, rf, ef, s);
}

ef_status ef_mpnn_num_samples(const ef_ctx* c, int* n) {
    if (!c || !n) return EF_ERR_ARG;
    int k = 0;
    for (const auto& S : c->nnSamples) k += S.sys >= 0;
    *n = k;
    return EF_OK;
}

ef_status ef_mpnn_clear_samples(ef_ctx* c) {
    EF_REQUIRE_FINALIZED(c);
    for (auto& S : c->nnSamples) S.sys = -1;
    for (auto& Y : c->nnSystems) Y.version = -1;
    c->nnAdded = 0;
    return EF_OK;
}

ef_status ef_mpnn_train(ef_ctx* c, int epochs, float lr, int norm, double* lossFirst, double* lossLast,
                        void* stream) {
    EF_REQUIRE_FINALIZED(c);
    if (epochs < 0 || !(lr >= 0.f) || norm < 0 || norm > 2) return EF_ERR_ARG;
    if (!c->nnInit) {
        ef_set_error("ef_mpnn_train: call ef_mpnn_init first");
        return EF_ERR_STATE;
    }
    return nn_train(c, epochs, lr, norm, lossFirst, lossLast, (cudaStream_t)stream);
}

ef_status ef_mpnn_eval(int nNodes, const int32_t* rowPtr, const int32_t* colIdx, const float* vals,
                       const float* params, const float* f, const float* base, const float* e, const uint8_t* mask,
                       float so, float scale, float* z, float* grad, double* loss, void* stream) {
    if (nNodes <= 0 || !rowPtr || !colIdx || !vals || !params || !f || !e || !z) return EF_ERR_ARG;
    cudaStream_t s = (cudaStream_t)stream;
    EF_CHECK(ef_mpnn_setup_kernels());
    const int64_t nN = nNodes, nb = rowPtr[nNodes], n = 3 * nN, H = ef_mpnn_hidden(), np = ef_mpnn_nparam();
    std::vector<int32_t> hr(rowPtr, rowPtr + nN + 1), hc(colIdx, colIdx + nb);
    for (int64_t m = 0; m < nN; ++m)
        if (hr[m + 1] < hr[m]) return EF_ERR_ARG;
    for (int32_t k : hc)
        if (k < 0 || k >= nNodes) return EF_ERR_ARG;
    std::vector<int64_t> tpos;
    EF_CHECK(nn_transpose_map(hr, hc, tpos));
    int dev = 0, nSM = 1;
    EF_CUDA(cudaGetDevice(&dev));
    EF_CUDA(cudaDeviceGetAttribute(&nSM, cudaDevAttrMultiProcessorCount, dev));
    const int nPart = 2 * nSM;
    ef_status st = EF_OK;
    std::vector<void*> owned;
    auto A = [&](size_t bytes) {
        void* p = nullptr;
        if (cudaMalloc(&p, bytes ? bytes : 1) != cudaSuccess) {
            st = EF_ERR_CUDA;
            return (void*)nullptr;
        }
        owned.push_back(p);
        return p;
    };
    int32_t* dR = (int32_t*)A(sizeof(int32_t) * (nN + 1));
    int32_t* dC = (int32_t*)A(sizeof(int32_t) * nb);
    float* dV = (float*)A(sizeof(float) * 9 * nb);
    float* dA = (float*)A(sizeof(float) * nb);
    float* dAT = (float*)A(sizeof(float) * nb);
    int64_t* dT = (int64_t*)A(sizeof(int64_t) * nb);
    float* dP = (float*)A(sizeof(float) * np);
    float* dF = (float*)A(sizeof(float) * 9 * nN);
    float* dB = base ? (float*)A(sizeof(float) * n) : nullptr;
    float* dE = (float*)A(sizeof(float) * n);
    uint8_t* dM = mask ? (uint8_t*)A(n) : nullptr;
    float* dZ = (float*)A(sizeof(float) * n);
    float* dG = (float*)A(sizeof(float) * np);
    float* acts = (float*)A(sizeof(float) * 10 * nN * H);
    float* work = (float*)A(sizeof(float) * 4 * nN * H);
    float* part = (float*)A(sizeof(float) * (size_t)nPart * H * H);
    double* red = (double*)A(sizeof(double) * (3 * nPart + 8));
    auto finish = [&](ef_status r) {
        for (void* p : owned) cudaFree(p);
        return r;
    };
    if (st != EF_OK) {
        ef_set_error("ef_mpnn_eval: cudaMalloc failed");
        return finish(st);
    }
#define EV_CUDA(x)                                                              \
    do {                                                                        \
        cudaError_t e_ = (x);                                                   \
        if (e_ != cudaSuccess) {                                                \
            ef_set_error(std::string("ef_mpnn_eval: ") + cudaGetErrorString(e_)); \
            return finish(EF_ERR_CUDA);                                         \
        }                                                                       \
    } while (0)
#define EV_CHECK(x)                   \
    do {                              \
        ef_status s_ = (x);           \
        if (s_ != EF_OK) return finish(s_); \
    } while (0)
    EV_CUDA(cudaMemcpyAsync(dR, hr.data(), sizeof(int32_t) * (nN + 1), cudaMemcpyHostToDevice, s));
    EV_CUDA(cudaMemcpyAsync(dC, hc.data(), sizeof(int32_t) * nb, cudaMemcpyHostToDevice, s));
    EV_CUDA(cudaMemcpyAsync(dV, vals, sizeof(float) * 9 * nb, cudaMemcpyHostToDevice, s));
    EV_CUDA(cudaMemcpyAsync(dT, tpos.data(), sizeof(int64_t) * nb, cudaMemcpyHostToDevice, s));
    EV_CUDA(cudaMemcpyAsync(dP, params, sizeof(float) * np, cudaMemcpyHostToDevice, s));
    EV_CUDA(cudaMemcpyAsync(dF, f, sizeof(float) * 9 * nN, cudaMemcpyHostToDevice, s));
    if (dB) EV_CUDA(cudaMemcpyAsync(dB, base, sizeof(float) * n, cudaMemcpyHostToDevice, s));
    EV_CUDA(cudaMemcpyAsync(dE, e, sizeof(float) * n, cudaMemcpyHostToDevice, s));
    if (dM) EV_CUDA(cudaMemcpyAsync(dM, mask, n, cudaMemcpyHostToDevice, s));
    EV_CHECK(ef_launch_edge_weights((int)nN, dR, dC, dV, dA, s));
    EV_CHECK(ef_launch_gather_f32(nb, dT, dA, dAT, s));
    EV_CHECK(ef_mpnn_forward((int)nN, dR, dC, dA, dP, dF, dB, dM, so, acts, dZ, 0, nullptr, s));
    EV_CHECK(ef_mpnn_sumsq(n, 1, dZ, dE, dM, red, nPart, red + 3 * nPart, s));
    if (grad)
        EV_CHECK(ef_mpnn_backward((int)nN, dR, dC, dAT, dP, dF, acts, dZ, dE, dM, scale, so, dG, work, part, nPart, s));
    EV_CUDA(cudaMemcpyAsync(z, dZ, sizeof(float) * n, cudaMemcpyDeviceToHost, s));
    if (grad) EV_CUDA(cudaMemcpyAsync(grad, dG, sizeof(float) * np, cudaMemcpyDeviceToHost, s));
    double l2 = 0.0;
    EV_CUDA(cudaMemcpyAsync(&l2, red + 3 * nPart, sizeof(double), cudaMemcpyDeviceToHost, s));
    EV_CUDA(cudaStreamSynchronize(s));
    if (loss) *loss = 0.5 * (double)scale * l2;
#undef EV_CUDA
#undef EV_CHECK
    return finish(EF_OK);
}

