// The FGMRES solve and ef_solve: the preconditioner application (multigrid cycle or block Jacobi,
// with the optional learned correction), FGMRES(m) with one-pass classical Gram-Schmidt, and the
// mixed-precision refinement loop around the inner PCG / FGMRES solves.

#include "ctx.h"

ef_status nn_apply(ef_ctx* c, cudaStream_t s) {
    const int64_t n = c->nDof;
    const int nN = (int)c->nNodes;
    const float* K = (const float*)c->dBsrVals;
    double* out = c->nnRed + 3 * c->nnPartN;
    EF_CHECK(ef_launch_spmv_f32(nN, c->dRowPtr, c->dColIdx, K, c->vcOut, c->dMask, c->nnKd, s));
    EF_CHECK(ef_launch_sub(n, c->vcIn, c->nnKd, c->nnRho, s));
    EF_CHECK(ef_launch_features(nN, c->vcOut, c->nnRho, (const float*)c->dBinv, c->nnS[0], c->nnS[1], c->nnS[2],
                                c->nnF, s));
    EF_CHECK(ef_mpnn_forward(nN, c->dRowPtr, c->dColIdx, c->nnA, c->nnPf, c->nnF, nullptr, c->dMask, c->nnSo,
                             c->nnActs, c->nnN, c->nnTensorCores, c->dFlags, s));
    EF_CHECK(ef_launch_spmv_f32(nN, c->dRowPtr, c->dColIdx, K, c->nnN, c->dMask, c->nnKN, s));
    EF_CHECK(ef_mpnn_sumsq(n, 0, c->nnRho, c->nnKN, c->dMask, c->nnRed, c->nnPartN, out, s));
    EF_CHECK(ef_mpnn_sumsq(n, 1, c->nnKN, nullptr, c->dMask, c->nnRed, c->nnPartN, out + 3, s));
    return ef_mpnn_alpha_combine(n, c->vcOut, c->nnN, out, c->dMask, c->vcOut2, s);
}

ef_status nn_capture(ef_ctx* c) {
    if (c->nnGraph) return EF_OK;
    if (!c->capStream) EF_CUDA(cudaStreamCreateWithFlags(&c->capStream, cudaStreamNonBlocking));
    EF_CUDA(cudaStreamBeginCapture(c->capStream, cudaStreamCaptureModeThreadLocal));
    long long captured = 0;
    t_captureCount = &captured;
    const ef_status st = nn_apply(c, c->capStream);
    t_captureCount = nullptr;
    c->nnGraphKernels = captured;
    cudaGraph_t g = nullptr;
    const cudaError_t e = cudaStreamEndCapture(c->capStream, &g);
    if (st != EF_OK) return st;
    if (e != cudaSuccess) {
        ef_set_error(std::string("network capture: ") + cudaGetErrorString(e));
        return EF_ERR_CUDA;
    }
    EF_CUDA(cudaGraphInstantiate(&c->nnGraph, g, 0));
    cudaGraphDestroy(g);
    return EF_OK;
}

// vcOut = M vcIn with the base preconditioner: the multigrid cycle (captured graph) or one
// block-Jacobi step D^-1 (free DOFs)
ef_status apply_base(ef_ctx* c, cudaStream_t s) {
    if (c->fgPc == EF_FGMRES_PC_JACOBI)
        return ef_launch_bj_apply(3, (int)c->nNodes, (const float*)c->dBinv, c->dMask, 1.f, c->vcIn, c->vcOut, 0, s);
    EF_CHECK(amg_capture(c));
    ef::note_launches(c->vcGraphKernels);
    EF_CUDA(cudaGraphLaunch(c->vcGraph, s));
    return EF_OK;
}

ef_status fgmres_precond(ef_ctx* c, const float* v, const float** out, cudaStream_t s) {
    if (c->vcInStale) {  // otherwise the previous column's normalisation wrote v into vcIn
        EF_CUDA(cudaMemcpyAsync(c->vcIn, v, sizeof(float) * c->nDof, cudaMemcpyDeviceToDevice, s));
        c->vcInStale = false;
    }
    EF_CHECK(apply_base(c, s));
    *out = c->vcOut;
    if (c->nnOn) {
        EF_CHECK(nn_edge_refresh(c, s, true));
        EF_CHECK(nn_capture(c));
        ef::note_launches(c->nnGraphKernels);
        EF_CUDA(cudaGraphLaunch(c->nnGraph, s));
        *out = c->vcOut2;
    }
    return EF_OK;
}

// ---- learned correction: weights, training pairs, training -----------------------------------

// deterministic normal variates (Box-Muller on a 64-bit Mersenne twister)
static ef_status run_fgmres(ef_ctx* c, const float* b, float* x, int maxIter, double rtol, int restart, int* iters,
                            ef_solve_info* prof, cudaStream_t s) {
    const int64_t n = c->nDof;
    const int m = std::max(2, std::min(restart, ef_fgmres_max_basis() - 2));
    ef_status st = EF_OK;
    if (c->fgRestart < m) {
        if (c->fgV) cudaFree(c->fgV);
        if (c->fgZ) cudaFree(c->fgZ);
        c->fgV = dalloc<float>((size_t)(m + 1) * n, &st);
        c->fgZ = dalloc<float>((size_t)m * n, &st);
        if (!c->fgV || !c->fgZ) return st;
        c->fgRestart = m;
    }
    if (!c->fgW) {
        c->fgW = dalloc<float>(n, &st);
        c->fgNPart = 4 * c->nSM;  // 1024 threads per SM
        c->fgPart = dalloc<double>((size_t)c->fgNPart * ef_fgmres_max_basis(), &st);
        c->fgPartN = dalloc<double>((size_t)c->fgNPart, &st);
        c->fgH = dalloc<double>(4 * (size_t)ef_fgmres_max_basis(), &st);
        if (!c->fgW || !c->fgPart || !c->fgPartN || !c->fgH) return st;
        c->fgPartF = dalloc<float>((size_t)c->nSM * ef_fgmres_max_basis(), &st);
        c->fgSc = dalloc<float>((size_t)ef_fgmres_max_basis(), &st);
        c->fgTicket = dalloc<unsigned>(1, &st);
        if (!c->fgPartF || !c->fgSc || !c->fgTicket) return st;
        EF_CUDA(cudaMemsetAsync(c->fgTicket, 0, sizeof(unsigned), s));
        if (const char* e = getenv("EF_FGMRES_ETA")) c->fgEta2 = atof(e) * atof(e);
        if (const char* e = getenv("EF_FGMRES_DEFER")) c->fgDefer = atoi(e) != 0;
        bool staged = false;  // measured slower than the unstaged kernel (EF_SPMV_STAGED=1 turns it on)
        if (const char* e = getenv("EF_SPMV_STAGED")) staged = atoi(e) != 0;
        c->spCap = staged ? ef_sp_stage_cap((int)c->nNodes, c->hRowPtr0.data()) : 0;
        if (c->spCap > 2048) c->spCap = 0;  // rows too long for a shared-memory stage
    }
    const int MB = ef_fgmres_max_basis();
    double* hG = c->fgH;            // first-pass coefficients and |w|^2 (the DGKS gate)
    double* hTmp = c->fgH + MB;     // second-pass coefficients
    double* hAcc = c->fgH + 2 * MB; // column of the Hessenberg matrix
    double* dy = c->fgH + 3 * MB;   // solution coefficients
    float* V = c->fgV;
    float* Z = c->fgZ;
    // Results of a column reach the host through mapped pinned memory written by the
    // normalisation kernel: [0, j] coefficients, ldh - 2 re-orthogonalised flag, ldh - 1 |w|^2.
    const int ldh = MB + 2;
    if (!c->fgPin) {
        EF_CUDA(cudaHostAlloc(&c->fgPin, sizeof(double) * 3 * ldh, cudaHostAllocMapped));
        EF_CUDA(cudaHostGetDevicePointer((void**)&c->fgPinDev, c->fgPin, 0));
        for (int k = 0; k < 2; ++k) {
            EF_CUDA(cudaEventCreateWithFlags(&c->fgDone[k], cudaEventDisableTiming));
        if (!c->fgNormDone) EF_CUDA(cudaEventCreateWithFlags(&c->fgNormDone, cudaEventDisableTiming));
            for (int e = 0; e < 4; ++e) EF_CUDA(cudaEventCreate(&c->fgEv[k][e]));
        }
    }
    double* pinRestart = c->fgPin + 2 * ldh;
    double* pinRestartDev = c->fgPinDev + 2 * ldh;
    const bool collect = c->nnInit && c->nnEvery > 0 && c->nnMaxPerSolve > 0;
    // deferred normalisation: needs the sliced-ELL product (it applies the factors) and one-pass
    // Gram-Schmidt; training samples are taken from normalised basis vectors, so not with them
    const bool defer = c->fgDefer && c->sellMode == 1 && !(c->fgEta2 > 0.0) && !collect;
    float* scRestart = defer ? c->fgSc : nullptr;
    EF_CUDA(cudaMemsetAsync(x, 0, sizeof(float) * n, s));
    // r0 = b (x = 0); v0 = r0 / |r0| (also into the preconditioner's input)
    EF_CUDA(cudaMemcpyAsync(V, b, sizeof(float) * n, cudaMemcpyDeviceToDevice, s));
    EF_CHECK(ef_launch_normalize_first(n, V, c->fgPart, c->fgNPart, c->vcIn, pinRestartDev, 0, s, scRestart));
    c->vcInStale = false;
    EF_CUDA(cudaEventRecord(c->fgNormDone, s));
    const bool snap = collect && c->nnKind == 0;
    const bool krylovSamples = collect && c->nnKind == 1;
    int nKrylov = 0;
    c->nnSnapCount = 0;
    if (snap) {  // x_0 = 0
        float* p = nullptr;
        EF_CHECK(nn_snapshot_buffer(c, &p));
        EF_CUDA(cudaMemsetAsync(p, 0, sizeof(float) * n, s));
    }
    std::vector<double> H((size_t)(m + 1) * m), cs(m), sn(m), g(m + 1);
    // The GPU work of column j+1 is enqueued before the host waits for column j's coefficients
    // (Givens rotations and the convergence test run on the host), so the GPU never idles on the
    // host; a converged cycle computes at most one column it does not use.
    auto enqueue_column = [&](int j) -> ef_status {
        const int sl = j & 1;
        if (prof) EF_CUDA(cudaEventRecord(c->fgEv[sl][0], s));
        const float* pz = nullptr;
        EF_CHECK(fgmres_precond(c, V + (int64_t)j * n, &pz, s));
        if (prof) EF_CUDA(cudaEventRecord(c->fgEv[sl][2], s));
        // w = K z_j straight into the next basis slot; z_j kept in Z
        if (c->sellMode == 1)
            EF_CHECK(ef_launch_sell_spmv3((int)c->nNodes, c->sellSlices, c->dSellOff, c->dSellPerm, c->dSellCol,
                                          c->dSellV9, pz, c->dMask, V + (int64_t)(j + 1) * n, Z + (int64_t)j * n,
                                          c->sellSplitProduct, s, defer ? c->fgSc + j : nullptr, c->dSellDia));
        else if (c->spCap > 0)
            EF_CHECK(ef_launch_spmv_f32_staged(c->nSM, c->spCap, (int)c->nNodes, c->dRowPtr, c->dColIdx,
                                               (const float*)c->dBsrVals, pz, c->dMask, V + (int64_t)(j + 1) * n,
                                               Z + (int64_t)j * n, s));
        else
            EF_CHECK(ef_launch_spmv_f32_copy((int)c->nNodes, c->dRowPtr, c->dColIdx, (const float*)c->dBsrVals, pz,
                                             c->dMask, V + (int64_t)(j + 1) * n, Z + (int64_t)j * n, s));
        if (prof) EF_CUDA(cudaEventRecord(c->fgEv[sl][3], s));
        if (defer)
            EF_CHECK(ef_launch_gs_column(n, j + 1, V, n, c->fgPartF, c->fgPartN, c->nSM, c->fgSc, c->fgTicket,
                                         c->vcIn, c->fgPinDev + sl * ldh, ldh - 1, s));
        else
            EF_CHECK(ef_launch_cgs_column(n, j + 1, V, n, c->fgPart, c->fgPartN, c->fgNPart, hG, hTmp, hAcc,
                                          c->fgEta2, c->vcIn, c->fgPinDev + sl * ldh, ldh - 1, s));
        c->vcInStale = false;
        if (prof) EF_CUDA(cudaEventRecord(c->fgEv[sl][1], s));
        EF_CUDA(cudaEventRecord(c->fgDone[sl], s));
        return EF_OK;
    };
    // column 0 runs while the host reads |b| (a zero b leaves every vector zero, and x = 0)
    EF_CHECK(enqueue_column(0));
    bool col0Queued = true;
    EF_CUDA(cudaEventSynchronize(c->fgNormDone));
    const double bnorm = sqrt(pinRestart[0]);
    *iters = 0;
    if (!(bnorm > 0.0)) {
        EF_CUDA(cudaStreamSynchronize(s));
        return EF_OK;
    }
    double beta = bnorm;
    int total = 0;
    bool converged = false;
    while (total < maxIter && !converged) {
        std::fill(g.begin(), g.end(), 0.0);
        g[0] = beta;
        int j = 0;
        if (!col0Queued) EF_CHECK(enqueue_column(0));
        col0Queued = false;
        // residual estimates after the last two columns: when the trend says column j reaches the
        // target (within the hold factor), column j + 1 is enqueued only once column j has been
        // read -- a short host turnaround instead of a whole column computed for nothing
        double res1 = -1.0, res2 = -1.0;
        for (; j < m && total < maxIter; ++j) {
            bool ahead = j + 1 < m && total + 1 < maxIter;
            if (ahead && res1 > 0.0 && res2 > 0.0 && res1 * (res1 / res2) <= c->fgHold * rtol * bnorm) ahead = false;
            if (ahead) EF_CHECK(enqueue_column(j + 1));
            const int sl = j & 1;
            EF_CUDA(cudaEventSynchronize(c->fgDone[sl]));
            const double* hcol = c->fgPin + sl * ldh;
            const double hn2 = hcol[ldh - 1];
            if (prof) {
                float ms = 0.f;
                EF_CUDA(cudaEventElapsedTime(&ms, c->fgEv[sl][0], c->fgEv[sl][1]));
                prof->kernelMs += ms;
                prof->kernelLaunches += 1;
                EF_CUDA(cudaEventElapsedTime(&ms, c->fgEv[sl][2], c->fgEv[sl][3]));
                prof->spmvMs += ms;
                prof->spmvLaunches += 1;
                EF_CUDA(cudaEventElapsedTime(&ms, c->fgEv[sl][0], c->fgEv[sl][2]));
                prof->precondMs += ms;
                EF_CUDA(cudaEventElapsedTime(&ms, c->fgEv[sl][3], c->fgEv[sl][1]));
                prof->orthoMs += ms;
            }
            if (prof && hcol[ldh - 2] != 0.0) prof->reorths += 1;
            ++total;
            double* Hj = &H[(size_t)j * (m + 1)];  // column j
            for (int i = 0; i <= j; ++i) Hj[i] = hcol[i];
            Hj[j + 1] = sqrt(hn2);
            for (int i = 0; i < j; ++i) {  // previous Givens rotations
                const double t0 = cs[i] * Hj[i] + sn[i] * Hj[i + 1];
                Hj[i + 1] = -sn[i] * Hj[i] + cs[i] * Hj[i + 1];
                Hj[i] = t0;
            }
            const double den = hypot(Hj[j], Hj[j + 1]);
            cs[j] = den > 0.0 ? Hj[j] / den : 1.0;
            sn[j] = den > 0.0 ? Hj[j + 1] / den : 0.0;
            Hj[j] = den;
            Hj[j + 1] = 0.0;
            g[j + 1] = -sn[j] * g[j];
            g[j] = cs[j] * g[j];
            if (!(g[j + 1] == g[j + 1]) || !(den == den)) {
                EF_CUDA(cudaStreamSynchronize(s));
                return EF_NAN;
            }
            if (krylovSamples && total % c->nnEvery == 0 && nKrylov < c->nnMaxPerSolve) {
                EF_CHECK(nn_add_sample(c, V + (int64_t)j * n, nullptr, s));
                ++nKrylov;
            }
            if (snap && total % c->nnEvery == 0 && c->nnSnapCount < c->nnMaxPerSolve && j + 1 < m) {
                // iterate after j + 1 steps: x + Z y, R y = g (current Givens factor)
                std::vector<double> ys(j + 1);
                for (int i = j; i >= 0; --i) {
                    double acc = g[i];
                    for (int k = i + 1; k <= j; ++k) acc -= H[(size_t)k * (m + 1) + i] * ys[k];
                    ys[i] = acc / H[(size_t)i * (m + 1) + i];
                }
                float* p = nullptr;
                EF_CHECK(nn_snapshot_buffer(c, &p));
                EF_CUDA(cudaMemcpyAsync(p, x, sizeof(float) * n, cudaMemcpyDeviceToDevice, s));
                EF_CUDA(cudaMemcpyAsync(dy, ys.data(), sizeof(double) * (j + 1), cudaMemcpyHostToDevice, s));
                EF_CHECK(ef_launch_combine(n, j + 1, Z, n, dy, p, s));
            }
            if (fabs(g[j + 1]) <= rtol * bnorm || hn2 <= 0.0) {
                converged = fabs(g[j + 1]) <= rtol * bnorm;
                ++j;
                break;
            }
            if (!ahead && j + 1 < m && total < maxIter) EF_CHECK(enqueue_column(j + 1));
            res2 = res1;
            res1 = fabs(g[j + 1]);
        }
        // y = R^-1 g, x += Z y
        std::vector<double> y(j);
        for (int i = j - 1; i >= 0; --i) {
            double acc = g[i];
            for (int k = i + 1; k < j; ++k) acc -= H[(size_t)k * (m + 1) + i] * y[k];
            y[i] = acc / H[(size_t)i * (m + 1) + i];
        }
        EF_CUDA(cudaMemcpyAsync(dy, y.data(), sizeof(double) * j, cudaMemcpyHostToDevice, s));
        EF_CHECK(ef_launch_combine(n, j, Z, n, dy, x, s));
        if (converged || total >= maxIter) break;
        // restart: r = b - K x
        EF_CHECK(ef_launch_spmv_f32((int)c->nNodes, c->dRowPtr, c->dColIdx, (const float*)c->dBsrVals, x, c->dMask,
                                    c->fineT, s));
        EF_CHECK(ef_launch_sub(n, b, c->fineT, V, s));
        EF_CHECK(ef_launch_normalize_first(n, V, c->fgPart, c->fgNPart, c->vcIn, pinRestartDev, 0, s, scRestart));
        c->vcInStale = false;
        EF_CUDA(cudaStreamSynchronize(s));
        beta = sqrt(pinRestart[0]);
        if (beta <= rtol * bnorm) {
            converged = true;
            break;
        }
    }
    *iters = total;
    if (snap && converged) EF_CHECK(nn_collect_snapshots(c, x, s));
    c->nnSnapCount = 0;
    return converged ? EF_OK : EF_NOT_CONVERGED;
}


ef_status ef_solve(ef_ctx* c, const ef_solve_opts* o, const double* b, double* x, ef_solve_info* info, void* stream) {
    EF_REQUIRE_FINALIZED(c);
    if (!o || !b || !x) return EF_ERR_ARG;
    if (o->method != EF_SOLVE_PCG && o->method != EF_SOLVE_FGMRES) {
        ef_set_error("ef_solve: unknown method");
        return EF_ERR_ARG;
    }
    if (o->method == EF_SOLVE_FGMRES && (c->keFp64 || !o->mixed)) {
        ef_set_error("ef_solve: FGMRES runs as the FP32 inner solver of the mixed-precision refinement");
        return EF_ERR_ARG;
    }
    if (!o->mixed && !c->keFp64) {
        ef_set_error("ef_solve: an all-FP64 solve needs an FP64 system (EF_OPT_KE_FP64)");
        return EF_ERR_ARG;
    }
    cudaStream_t s = (cudaStream_t)stream;
    const int64_t n = c->nDof;
    double* xd = c->w64[0];
    double* xf = c->w64[1];
    double* r64 = c->w64[2];
    double* tmp = c->w64[3];
    ef_solve_info inf;
    memset(&inf, 0, sizeof(inf));
    inf.status = EF_OK;
    double bb = 0.0;
    EF_CHECK(dot_host(c, b, b, &bb, s));
    // Dirichlet part: x_d = b on Dirichlet DOFs; lifted RHS b~ = b_f - K_fd x_d (when x_d = 0, as in
    // every Newton system after an increment's first, b~ is b on the free DOFs: the same bits
    // without the operator application)
    EF_CHECK(ef_launch_masked_copy(n, b, c->dMask, 1, 1.0, xd, 1, s));
    double dd = 0.0;
    EF_CHECK(dot_host(c, xd, xd, &dd, s));
    if (dd == 0.0)
        EF_CHECK(ef_launch_masked_copy(n, b, c->dMask, 0, 1.0, r64, 1, s));
    else
        EF_CHECK(residual64(c, xd, b, r64, s));
    EF_CUDA(cudaMemsetAsync(xf, 0, sizeof(double) * n, s));
    if (!(bb > 0.0)) {
        EF_CUDA(cudaMemsetAsync(x, 0, sizeof(double) * n, s));
        inf.relResidual = 0.0;
        if (info) *info = inf;
        return EF_OK;
    }
    const double bnorm = sqrt(bb);
    double rr = 0.0;
    EF_CHECK(dot_host(c, r64, r64, &rr, s));
    int total = 0;
    ef_status result = EF_OK;
    if (!o->mixed) {
        // all-FP64 PCG to the target tolerance (relative to ||b||)
        EF_CUDA(cudaMemcpyAsync(c->w64k[0], r64, sizeof(double) * n, cudaMemcpyDeviceToDevice, s));
        const double rel = rr > 0.0 ? o->rtol * bnorm / sqrt(rr) : 1.0;
        PcgResultHost pr;
        if (rr > 0.0) {
            EF_CHECK(run_pcg(c, 1, c->w64k[0], c->w64k[1], o->maxIter, std::min(rel, 1.0), &pr, o->profile ? &inf : nullptr, s));
            total = pr.iterations;
            if (pr.status == EF_NAN) result = EF_NAN;
            EF_CHECK(ef_launch_axpy(n, 1.0, c->w64k[1], 1, xf, s));
        }
    } else {
        for (int sweep = 0; sweep < o->maxRefine; ++sweep) {
            if (!(rr == rr)) {
                result = EF_NAN;
                break;
            }
            if (sqrt(rr) <= o->rtol * bnorm) break;
            if (total >= o->maxIter) break;
            const double rn = sqrt(rr);
            // inner solve of K d = r / ||r|| in the system's precision (FP32 unless EF_OPT_KE_FP64)
            const int vd = c->keFp64;
            void** wv = vd ? c->w64k : c->w32;
            EF_CHECK(ef_launch_masked_copy(n, r64, c->dMask, 0, 1.0 / rn, wv[0], vd, s));
            // the first inner solve to innerRtol; with the multigrid-preconditioned FGMRES the later
            // ones no tighter than what such an FP32 solve lowers the FP64 residual by (refineFloor,
            // measured), nor than the remaining target needs
            const bool floored = sweep > 0 && o->method == EF_SOLVE_FGMRES &&
                                 c->fgPc == EF_FGMRES_PC_MULTIGRID && !c->nnOn;
            const double inner = std::max(floored ? std::max(o->innerRtol, c->refineFloor) : o->innerRtol,
                                          c->refineAim * o->rtol * bnorm / rn);
            PcgResultHost pr;
            if (o->method == EF_SOLVE_FGMRES) {
                const bool timeSetup = o->profile && (c->sellStale || c->amgStale);
                if (timeSetup) EF_CUDA(cudaEventRecord(c->ev[0], s));
                EF_CHECK(sell_refresh(c, s));
                if (c->fgPc == EF_FGMRES_PC_MULTIGRID) {
                    EF_CHECK(amg_build(c));
                    EF_CHECK(amg_refresh(c, s));
                } else {
                    EF_CHECK(amg_workspace(c));
                    EF_CHECK(nn_edge_refresh(c, s));
                }
                if (timeSetup) {
                    EF_CUDA(cudaEventRecord(c->ev[1], s));
                    EF_CUDA(cudaEventSynchronize(c->ev[1]));
                    float ms = 0.f;
                    EF_CUDA(cudaEventElapsedTime(&ms, c->ev[0], c->ev[1]));
                    inf.setupMs += ms;
                }
                int its = 0;
                const ef_status fs = run_fgmres(c, (const float*)wv[0], (float*)wv[1], o->maxIter - total,
                                                std::min(inner, 0.5), o->restart, &its, o->profile ? &inf : nullptr, s);
                if (fs != EF_OK && fs != EF_NOT_CONVERGED && fs != EF_NAN) return fs;
                pr.iterations = its;
                pr.status = fs;
                pr.rr = 0.0;
                pr.bb = 0.0;
            } else {
                EF_CHECK(run_pcg(c, vd, wv[0], wv[1], o->maxIter - total, std::min(inner, 0.5), &pr,
                                 o->profile ? &inf : nullptr, s));
            }
            total += pr.iterations;
            inf.refinements++;
            if (pr.status == EF_NAN) {
                result = EF_NAN;
                break;
            }
            if (pr.iterations == 0) break;  // no progress possible
            EF_CHECK(ef_launch_axpy(n, rn, wv[1], vd, xf, s));
            // r64 = b~ - K x_f  (FP64 accumulation); b~ = b - K x_d on free rows
            EF_CHECK(ef_launch_add(n, xd, xf, tmp, s));
            EF_CHECK(residual64(c, tmp, b, r64, s));
            EF_CHECK(dot_host(c, r64, r64, &rr, s));
        }
    }
    EF_CHECK(ef_launch_add(n, xd, xf, x, s));
    if (c->dTieS) EF_CHECK(ef_launch_tie_fill((int64_t)c->hTieS.size(), c->dTieS, c->dTieA, c->dTieB, x, s));
    // final FP64 residual of the full system (Dirichlet rows are exact); the refinement loop
    // leaves r64 = b - K (x_d + x_f) of this very x (every exit follows a residual of the current
    // x_f), so it is recomputed only after the all-FP64 solve and where tied DOFs were filled
    if (!o->mixed || c->dTieS) {
        EF_CHECK(residual64(c, x, b, r64, s));
        EF_CHECK(dot_host(c, r64, r64, &rr, s));
    }
    inf.iterations = total;
    inf.relResidual = sqrt(rr) / bnorm;
    if (result == EF_OK && !(inf.relResidual <= o->rtol)) result = (rr == rr) ? EF_NOT_CONVERGED : EF_NAN;
    inf.status = result;
    if (info) *info = inf;
    if (o->method == EF_SOLVE_FGMRES && c->nnOn && c->nnTensorCores) {
        // a tensor-core tile that gave up waiting freed its TMEM while its MMA may still have been
        // running: the solve that used the network is discarded and the network continues on
        // the CUDA-core layer for the rest of this context
        int f = 0;
        EF_CUDA(cudaMemcpy(&f, c->dFlags, sizeof(int), cudaMemcpyDeviceToHost));
        if (f & EF_FLAG_TCWAIT) {
            EF_CUDA(cudaMemset(c->dFlags, 0, sizeof(int)));
            c->nnTensorCores = 0;
            if (c->nnGraph) {  // the captured network pass holds the tensor-core layer: capture again
                cudaGraphExecDestroy(c->nnGraph);
                c->nnGraph = nullptr;
            }
            ef_set_error("ef_solve: the learned correction's tensor-core accumulator wait timed out; this solve is "
                         "discarded and the network runs on the CUDA cores from now on");
            if (info) info->status = EF_ERR_DEVICE;
            return EF_ERR_DEVICE;
        }
    }
    return result;
}

ef_status ef_fine_kernel_profile(ef_ctx* c, int reps, double* ms, double* bytes, void* stream) {
    EF_REQUIRE_FINALIZED(c);
    if (reps < 1 || !ms || !bytes) return EF_ERR_ARG;
    if (c->sellMode != 1 || !c->dSellV8 || !c->vcIn || !c->vcOut || !c->fineX || !c->fineT || !c->fgZ) {
        ef_set_error("ef_fine_kernel_profile: needs an FGMRES solve with the sliced-ELL fine level first");
        return EF_ERR_STATE;
    }
    cudaStream_t s = (cudaStream_t)stream;
    const int nN = (int)c->nNodes;
    const float omega = c->levelOmega.empty() ? c->amgOmega : c->levelOmega[0];
    // the fine residual as the cycle runs it: t = r - w K (M D^-1) r from the scaled copy, or a
    // damped sweep from the plain one
    auto sweep = [&]() {
        if (c->sellScaled)
            return ef_launch_sell_level3_bf16(nN, c->sellSlices, c->dSellOff, c->dSellPerm, c->dSellCol, c->dSellV8,
                                              c->dSellV1, c->vcIn, c->vcIn, c->dMask, c->fineT, nullptr, 0.f,
                                              c->sellSplit, s, omega, c->dSellDia);
        return ef_launch_sell_level3_bf16(nN, c->sellSlices, c->dSellOff, c->dSellPerm, c->dSellCol, c->dSellV8,
                                          c->dSellV1, c->fineX, c->vcIn, c->dMask, c->fineT, (const float*)c->dBinv,
                                          omega, c->sellSplit, s, 1.f, c->dSellDia);
    };
    auto product = [&]() {
        return ef_launch_sell_spmv3(nN, c->sellSlices, c->dSellOff, c->dSellPerm, c->dSellCol, c->dSellV9, c->vcOut,
                                    c->dMask, c->fineT, c->fgZ, c->sellSplitProduct, s, nullptr, c->dSellDia);
    };
    const bool post = c->postSlots > 0 && !c->amg.empty() && c->amg[0].x;
    auto fused = [&]() {
        return ef_launch_sa_post_fused(nN, c->postSlices, c->dPostOff, c->dPostPerm, c->dPostCol, c->dPostQ0,
                                       c->dPostQ1, c->dPostQ2, c->amg[0].x, c->vcIn, c->fineT, (const float*)c->dBinv,
                                       c->dMask, omega, c->fineX, c->sellSplit, s);
    };
    for (int k = 0; k < 3; ++k) {
        ms[k] = 0.0;
        if (k == 2 && !post) continue;
        auto run = [&]() { return k == 0 ? sweep() : (k == 1 ? product() : fused()); };
        EF_CHECK(run());  // warm-up
        EF_CUDA(cudaEventRecord(c->ev[0], s));
        for (int i = 0; i < reps; ++i) EF_CHECK(run());
        EF_CUDA(cudaEventRecord(c->ev[1], s));
        EF_CUDA(cudaEventSynchronize(c->ev[1]));
        float t = 0.f;
        EF_CUDA(cudaEventElapsedTime(&t, c->ev[0], c->ev[1]));
        ms[k] = (double)t / reps;
    }
    // algorithmic DRAM bytes per launch: the real blocks (values and column indices; the slices'
    // padding is layout overhead, 3.9 % on the structured box) and the per-row vectors
    // (the diagonal form reads no column indices: 4 bytes less per block)
    const double nb = (double)c->nBlocks, nn = (double)nN, ns = (double)c->sellSlices;
    const double colB = c->dSellDia ? 0.0 : 4.0;
    bytes[0] = nb * (16 + 2 + colB) + nn * (3 * 4 /*x*/ + 3 * 4 /*r*/ + 9 * 4 /*D^-1*/ + 3 /*mask*/ + 3 * 4 /*out*/) +
               (ns + 1) * 8;
    if (c->sellScaled) bytes[0] -= nn * (3 * 4 /*x*/ + 9 * 4 /*D^-1*/);  // x is r, no D^-1 in the residual
    bytes[1] = nb * (9 * 4 + colB) + nn * (3 * 4 /*x*/ + 3 /*mask*/ + 3 * 4 /*y*/ + 3 * 4 /*copy*/) + (ns + 1) * 8;
    // the fused post-smoothing: C blocks (18 BF16 values and a column) of the pattern of A P, the
    // per-row r, t, D^-1, mask and output (the coarse correction e, 40 k values, is read from cache)
    bytes[2] = post ? (double)c->amg[0].saNAP * (18 * 2 + 4) +
                          nn * (3 * 4 /*r*/ + 3 * 4 /*t*/ + 9 * 4 /*D^-1*/ + 3 /*mask*/ + 3 * 4 /*out*/) +
                          (double)(c->postSlices + 1) * 8
                    : 0.0;
    return EF_OK;
}

ef_status ef_fgmres_set_reuse(ef_ctx* c, int maxReuse) {
    EF_REQUIRE_FINALIZED(c);
    if (maxReuse < 0) {
        ef_set_error("ef_fgmres_set_reuse: maxReuse must be >= 0");
        return EF_ERR_ARG;
    }
    c->amgMaxReuse = maxReuse;
    c->amgReuseLeft = 0;    // the next new system rebuilds the coarse levels
    c->amgPowerDue = true;  // and re-estimates the damping
    return EF_OK;
}

ef_status ef_fgmres_set_preconditioner(ef_ctx* c, int kind) {
    EF_REQUIRE_FINALIZED(c);
    if (kind != EF_FGMRES_PC_MULTIGRID && kind != EF_FGMRES_PC_JACOBI) {
        ef_set_error("ef_fgmres_set_preconditioner: unknown kind");
        return EF_ERR_ARG;
    }
    if (kind != c->fgPc && c->nnGraph) {  // the correction's captured graph reads the base output
        cudaGraphExecDestroy(c->nnGraph);
        c->nnGraph = nullptr;
    }
    c->fgPc = kind;
    return EF_OK;
}

