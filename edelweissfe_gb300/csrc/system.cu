// C ABI of the assembled system: the reference-layout VIJ values and scalar CSR, the Dirichlet
// set, the 3x3-block assembly, its FP64 product and residual, the block-Jacobi PCG runner, the
// convergence reductions and the device Newton check.

#include "ctx.h"

ef_status ef_export_vij(ef_ctx* c, double* Kvij, void* stream) {
    EF_REQUIRE_FINALIZED(c);
    if (!Kvij) return EF_ERR_ARG;
    const size_t ks = c->keFp64 ? sizeof(double) : sizeof(float);
    int64_t vijOff = 0;
    for (const auto& g : c->groups) {
        const void* K = (const char*)c->Kblk + (size_t)g.keOffset * 9 * ks;
        EF_CHECK(ef_launch_vij_export(g.nEl, g.nNodes, g.nPair, K, c->keFp64, Kvij + vijOff, (cudaStream_t)stream));
        vijOff += (int64_t)g.nEl * g.nDofEl * g.nDofEl;
    }
    return EF_OK;
}

ef_status ef_csr_pattern(ef_ctx* c, int32_t* indptr, int32_t* indices) {
    EF_REQUIRE_FINALIZED(c);
    if (!c->scalar) {
        ef_set_error("ef_csr_pattern: context finalized with EF_OPT_NO_SCALAR_CSR");
        return EF_ERR_STATE;
    }
    if (indptr) EF_CUDA(cudaMemcpy(indptr, c->hIndptr.data(), sizeof(int32_t) * (c->nDof + 1), cudaMemcpyDefault));
    if (indices) EF_CUDA(cudaMemcpy(indices, c->hIndices.data(), sizeof(int32_t) * c->nnz, cudaMemcpyDefault));
    return EF_OK;
}

ef_status ef_update_csr(ef_ctx* c, const double* Kvij, double* csrData, void* stream) {
    EF_REQUIRE_FINALIZED(c);
    if (!c->scalar || !csrData) {
        ef_set_error("ef_update_csr: no scalar CSR map or null output");
        return EF_ERR_STATE;
    }
    cudaStream_t s = (cudaStream_t)stream;
    if (!Kvij) {
        if (!c->dKvijTmp) {
            ef_status st = EF_OK;
            c->dKvijTmp = dalloc<double>(c->nVIJ, &st);
            if (!c->dKvijTmp) return st;
        }
        EF_CHECK(ef_export_vij(c, c->dKvijTmp, stream));
        Kvij = c->dKvijTmp;
    }
    return ef_launch_csr_scatter(c->nnz, c->dCsrSeg, c->dCsrPerm, Kvij, csrData, s);
}

ef_status ef_csr_dirichlet_rows(ef_ctx* c, double* csrData, const int64_t* rows, int64_t nRows, void* stream) {
    EF_REQUIRE_FINALIZED(c);
    if (!c->scalar || !csrData || (nRows > 0 && !rows)) return EF_ERR_ARG;
    if (nRows == 0) return EF_OK;
    for (int64_t i = 0; i < nRows; ++i)
        if (rows[i] < 0 || rows[i] >= c->nDof) {
            ef_set_error("ef_csr_dirichlet_rows: row out of range");
            return EF_ERR_ARG;
        }
    ef_status st = EF_OK;
    int64_t* d = dalloc<int64_t>(nRows, &st);
    if (!d) return st;
    cudaStream_t s = (cudaStream_t)stream;
    cudaMemcpyAsync(d, rows, sizeof(int64_t) * nRows, cudaMemcpyHostToDevice, s);
    st = ef_launch_csr_dirichlet_rows(nRows, d, c->dIndptr, c->dIndices, csrData, s);
    cudaStreamSynchronize(s);
    cudaFree(d);
    return st;
}

ef_status ef_set_dirichlet(ef_ctx* c, const int64_t* dofs, int64_t n) {
    EF_REQUIRE_FINALIZED(c);
    std::vector<uint8_t> m(c->nDof, 0);
    for (int64_t i = 0; i < n; ++i) {
        if (dofs[i] < 0 || dofs[i] >= c->nDof) {
            ef_set_error("ef_set_dirichlet: DOF out of range");
            return EF_ERR_ARG;
        }
        m[dofs[i]] = 1;
    }
    {
        ef_status st = EF_OK;
        if (c->dDirIdx) cudaFree(c->dDirIdx);
        if (c->dDirMask) cudaFree(c->dDirMask);
        c->dDirIdx = nullptr;
        c->dDirMask = nullptr;
        c->nDir = n;
        if (n > 0) {
            c->dDirIdx = dalloc<int64_t>((size_t)n, &st);
            if (!c->dDirIdx) return st;
            EF_CUDA(cudaMemcpy(c->dDirIdx, dofs, sizeof(int64_t) * n, cudaMemcpyHostToDevice));
        }
        c->dDirMask = dalloc<uint8_t>((size_t)c->nDof, &st);
        if (!c->dDirMask) return st;
        EF_CUDA(cudaMemcpy(c->dDirMask, m.data(), c->nDof, cudaMemcpyHostToDevice));
    }
    for (int32_t sN : c->hTieS)
        for (int k = 0; k < 3; ++k) m[3 * (int64_t)sN + k] = 1;
    c->anyDirichlet = n > 0 || !c->hTieS.empty();
    EF_CUDA(cudaMemcpy(c->dMask, m.data(), c->nDof, cudaMemcpyHostToDevice));
    c->hMask = std::move(m);
    c->amgStale = true;
    c->amgMaskChanged = true;
    c->amgPowerDue = true;
    c->nnEdgeStale = true;
    c->nnVersion++;
    return EF_OK;
}

ef_status ef_assemble_bsr(ef_ctx* c, void* stream) {
    EF_REQUIRE_FINALIZED(c);
    cudaStream_t s = (cudaStream_t)stream;
    c->sellStale = true;
    EF_CHECK(ef_launch_bsr_scatter(c->nBlocks, c->dBsrSeg, c->dBsrSrc, c->dBsrW, c->Kblk, c->keFp64, c->dBsrVals, s));
    EF_CHECK(ef_launch_bj_setup(c->nNodes, c->dDiagPos, c->dNodeDof, c->dMask, c->dBsrVals, c->keFp64, c->dBinv,
                                c->dFlags, s));
    c->amgStale = true;
    c->nnEdgeStale = true;
    c->nnVersion++;
    return EF_OK;
}

ef_status ef_bsr_matvec(ef_ctx* c, const double* x, double* y, void* stream) {
    EF_REQUIRE_FINALIZED(c);
    return ef_launch_bsr_residual((int)c->nNodes, c->dRowPtr, c->dColIdx, c->dBsrVals, c->keFp64, x, nullptr,
                                  c->anyDirichlet ? c->dMask : nullptr, y, c->nSM, (cudaStream_t)stream);
}

// r = b - K x on free rows (0 on Dirichlet rows): with the exact FP64 tangent (matrix-free element
// apply) when the system is stored in FP32, else with the stored system
ef_status residual64(ef_ctx* c, const double* x, const double* b, double* r, cudaStream_t s) {
    if (!c->exact)
        return ef_launch_bsr_residual((int)c->nNodes, c->dRowPtr, c->dColIdx, c->dBsrVals, c->keFp64, x, b, c->dMask,
                                      r, c->nSM, s);
    double* y = c->w64[4];
    if (c->dTieS) {  // the element apply needs the tied DOFs filled from their masters
        EF_CUDA(cudaMemcpyAsync(c->dTieTmp, x, sizeof(double) * c->nDof, cudaMemcpyDeviceToDevice, s));
        EF_CHECK(ef_launch_tie_fill((int64_t)c->hTieS.size(), c->dTieS, c->dTieA, c->dTieB, c->dTieTmp, s));
        x = c->dTieTmp;
    }
    for (size_t gi = 0; gi < c->groups.size(); ++gi) {
        const Group& g = c->groups[gi];
        if (g.tl)
            EF_CHECK(ef_launch_total_lagrange_apply(g, x, c->dTang[gi], c->dYe + g.peOffset, s));
        else
            EF_CHECK(ef_launch_small_strain_apply(g, x, c->dTang[gi], c->dYe + g.peOffset, s));
    }
    EF_CHECK(ef_launch_condense(c->nNodes, c->dNodeDof, c->dCondPtr, c->dCondSrc, c->dCondW, c->dYe, y, nullptr, s));
    return ef_launch_residual_from(c->nDof, b, y, c->dMask, r, s);
}

ef_status dot_host(ef_ctx* c, const double* a, const double* b, double* out, cudaStream_t s) {
    EF_CHECK(ef_launch_dot(c->nDof, a, b, c->dPart, c->nPart, c->dRed, s));
    EF_CUDA(cudaMemcpyAsync(out, c->dRed, sizeof(double), cudaMemcpyDeviceToHost, s));
    EF_CUDA(cudaStreamSynchronize(s));
    return EF_OK;
}

// one PCG launch on the free DOFs: solves K d = rhs (rhs zero on Dirichlet DOFs)
ef_status run_pcg(ef_ctx* c, int vDouble, const void* rhs, void* sol, int maxIter, double rtol,
                         PcgResultHost* out, ef_solve_info* prof, cudaStream_t s) {
    void** w = vDouble ? c->w64k : c->w32;
    EF_CUDA(cudaMemsetAsync(c->dBar, 0, ef_barrier_state_bytes(), s));
    if (prof) EF_CUDA(cudaEventRecord(c->ev[0], s));
    EF_CHECK(ef_launch_pcg(vDouble, c->pcgGrid[vDouble], (int)c->nNodes, c->dRowPtr, c->dColIdx, c->dBsrVals, c->dBinv,
                           c->dMask, rhs, sol, w[2], w[3], w[4], w[5], w[6], c->dPartA, c->dPartB, c->dBar,
                           c->dPcgRes, maxIter, rtol * rtol, c->dFlags, s));
    if (prof) EF_CUDA(cudaEventRecord(c->ev[1], s));
    EF_CUDA(cudaMemcpyAsync(out, c->dPcgRes, sizeof(PcgResultHost), cudaMemcpyDeviceToHost, s));
    EF_CUDA(cudaStreamSynchronize(s));
    if (prof) {
        float ms = 0.f;
        EF_CUDA(cudaEventElapsedTime(&ms, c->ev[0], c->ev[1]));
        prof->kernelMs += ms;
        prof->kernelLaunches += 1;
    }
    int f = 0;
    EF_CUDA(cudaMemcpy(&f, c->dFlags, sizeof(int), cudaMemcpyDeviceToHost));
    if (f & EF_FLAG_BARRIER) {
        ef_set_error("PCG: grid barrier timed out");
        return EF_ERR_DEVICE;
    }
    return EF_OK;
}



ef_status ef_newton_residual(ef_ctx* c, int mode, const double* P, const double* PExt, const double* dirValues,
                             const double* F, const double* ddU, int iteration, double prevResidual, int nGrew,
                             const ef_newton_opts* o, double* R, ef_newton_check* out, void* stream) {
    EF_REQUIRE_FINALIZED(c);
    if (!P || !R || (mode != 0 && mode != 1) || (mode == 1 && (!F || !o || !out)) ||
        (mode == 0 && c->nDir > 0 && !dirValues)) {
        ef_set_error("ef_newton_residual: bad arguments");
        return EF_ERR_ARG;
    }
    if (!c->dDirMask) {
        ef_set_error("ef_newton_residual: call ef_set_dirichlet first");
        return EF_ERR_STATE;
    }
    cudaStream_t s = (cudaStream_t)stream;
    if (mode == 0) return ef_launch_newton_first(c->nDof, P, PExt, c->nDir, c->dDirIdx, dirValues, R, s);
    if (!c->dNewton) {
        ef_status st = EF_OK;
        c->dNewton = dalloc<double>(16, &st);
        if (!c->dNewton) return st;
    }
    const double q[9] = {o->fluxTol, o->fluxTolAlt, o->corrTol, o->fluxFloor, o->nAccFluxes, prevResidual,
                         (double)iteration, (double)nGrew, ddU ? 1.0 : 0.0};
    EF_CUDA(cudaMemcpyAsync(c->dNewton, q, sizeof(q), cudaMemcpyHostToDevice, s));
    EF_CHECK(ef_launch_newton_check(c->nDof, P, PExt, c->dDirMask, F, ddU, R, c->dPart, c->nPart, c->dNewton,
                                    c->dNewton + 9, s));
    double r[5];
    EF_CUDA(cudaMemcpyAsync(r, c->dNewton + 9, sizeof(r), cudaMemcpyDeviceToHost, s));
    EF_CUDA(cudaStreamSynchronize(s));
    out->converged = r[0] != 0.0;
    out->nGrew = (int)r[1];
    out->fluxResidual = r[2];
    out->fieldCorrection = r[3];
    out->spatialAveragedFlux = r[4];
    return EF_OK;
}

ef_status ef_norms(ef_ctx* c, const double* R, const double* F, const double* ddU, double* out, void* stream) {
    EF_REQUIRE_FINALIZED(c);
    if (!out) return EF_ERR_ARG;
    cudaStream_t s = (cudaStream_t)stream;
    EF_CHECK(ef_launch_norms(c->nDof, R, F, ddU, c->dPart, c->nPart, c->dRed, s));
    EF_CUDA(cudaMemcpyAsync(out, c->dRed, 3 * sizeof(double), cudaMemcpyDeviceToHost, s));
    EF_CUDA(cudaStreamSynchronize(s));
    return EF_OK;
}

