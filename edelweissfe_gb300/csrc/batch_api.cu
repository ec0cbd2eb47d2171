// C ABI of batches of independent problems in one context: problem ranges, tile shapes and their
// autotuner, the one-launch batched PCG and per-problem norms.

#include "ctx.h"

ef_status ef_batch_setup(ef_ctx* c, int nProb, const int32_t* nodePtr) {
    EF_REQUIRE_FINALIZED(c);
    if (nProb <= 0 || !nodePtr || nodePtr[0] != 0 || nodePtr[nProb] != (int32_t)c->nNodes) {
        ef_set_error("ef_batch_setup: node ranges must cover [0, nNodes)");
        return EF_ERR_ARG;
    }
    for (int p = 0; p < nProb; ++p)
        if (nodePtr[p + 1] < nodePtr[p]) {
            ef_set_error("ef_batch_setup: node ranges must be increasing");
            return EF_ERR_ARG;
        }
    if (!c->keFp64) {
        ef_set_error("ef_batch_setup: the batched solve runs on the FP64 system (EF_OPT_KE_FP64)");
        return EF_ERR_ARG;
    }
    // every block must couple nodes of one problem (block-diagonal system)
    std::vector<int32_t> prob(c->nNodes);
    for (int p = 0; p < nProb; ++p)
        for (int32_t m = nodePtr[p]; m < nodePtr[p + 1]; ++m) prob[m] = p;
    for (int64_t m = 0; m < c->nNodes; ++m)
        for (int32_t k = c->hRowPtr0[m]; k < c->hRowPtr0[m + 1]; ++k)
            if (prob[c->hColIdx0[k]] != prob[m]) {
                ef_set_error("ef_batch_setup: a block couples two problems");
                return EF_ERR_ARG;
            }
    std::vector<int32_t> order(nProb);
    for (int p = 0; p < nProb; ++p) order[p] = p;
    std::stable_sort(order.begin(), order.end(), [&](int32_t a, int32_t b) {
        return nodePtr[a + 1] - nodePtr[a] > nodePtr[b + 1] - nodePtr[b];
    });
    if (c->dBatchNodePtr) cudaFree(c->dBatchNodePtr);
    if (c->dBatchOrder) cudaFree(c->dBatchOrder);
    ef_status st = EF_OK;
    c->dBatchNodePtr = dalloc<int32_t>(nProb + 1, &st);
    c->dBatchOrder = dalloc<int32_t>(nProb, &st);
    if (st != EF_OK) return st;
    EF_CUDA(cudaMemcpy(c->dBatchNodePtr, nodePtr, sizeof(int32_t) * (nProb + 1), cudaMemcpyHostToDevice));
    EF_CUDA(cudaMemcpy(c->dBatchOrder, order.data(), sizeof(int32_t) * nProb, cudaMemcpyHostToDevice));
    c->batchN = nProb;
    return EF_OK;
}

ef_status ef_batch_set_tile(ef_ctx* c, int tile) {
    EF_REQUIRE_FINALIZED(c);
    if (tile < 0 || tile >= ef_batch_num_tiles()) {
        ef_set_error("ef_batch_set_tile: unknown tile shape");
        return EF_ERR_ARG;
    }
    c->batchTile = tile;
    return EF_OK;
}

int ef_batch_tile_count(void) { return ef_batch_num_tiles(); }

ef_status ef_batch_tile_info(int tile, int* threadsPerCta, int* lanesPerRow) {
    if (tile < 0 || tile >= ef_batch_num_tiles() || !threadsPerCta || !lanesPerRow) return EF_ERR_ARG;
    ef_batch_tile_shape(tile, threadsPerCta, lanesPerRow);
    return EF_OK;
}

static ef_status batch_solve(ef_ctx* c, int tile, double rtol, int maxIter, const double* b, double* x, int* iters,
                             double* relres, cudaStream_t s) {
    const int64_t n = c->nDof;
    double* xd = c->w64[0];
    double* r64 = c->w64[2];
    // Dirichlet DOFs take b; the free part solves K_ff x_f = b_f - K_fd x_d per problem
    EF_CHECK(ef_launch_masked_copy(n, b, c->dMask, 1, 1.0, xd, 1, s));
    EF_CHECK(residual64(c, xd, b, r64, s));
    double* w[5];
    for (int i = 0; i < 5; ++i) w[i] = (double*)c->w64k[1 + i];
    EF_CHECK(ef_launch_batched_pcg(tile, c->nSM, c->batchN, c->dBatchNodePtr, c->dBatchOrder, c->dRowPtr, c->dColIdx,
                                   (const double*)c->dBsrVals, (const double*)c->dBinv, c->dMask, r64, w[0], w[1],
                                   w[2], w[3], w[4], maxIter, rtol * rtol, iters, relres, s));
    return ef_launch_add(n, xd, w[0], x, s);
}

ef_status ef_batch_solve(ef_ctx* c, double rtol, int maxIter, const double* b, double* x, int* iters, double* relres,
                         void* stream) {
    EF_REQUIRE_FINALIZED(c);
    if (c->batchN == 0) {
        ef_set_error("ef_batch_solve: call ef_batch_setup first");
        return EF_ERR_STATE;
    }
    if (!b || !x || !iters || !relres || !(rtol > 0.0) || maxIter < 0) return EF_ERR_ARG;
    return batch_solve(c, c->batchTile, rtol, maxIter, b, x, iters, relres, (cudaStream_t)stream);
}

ef_status ef_batch_autotune(ef_ctx* c, double rtol, int maxIter, const double* b, double* x, int* iters,
                            double* relres, void* stream, int* tileOut, float* msOut) {
    EF_REQUIRE_FINALIZED(c);
    if (c->batchN == 0) {
        ef_set_error("ef_batch_autotune: call ef_batch_setup first");
        return EF_ERR_STATE;
    }
    cudaStream_t s = (cudaStream_t)stream;
    float best = 1e30f;
    int bestT = c->batchTile;
    for (int t = 0; t < ef_batch_num_tiles(); ++t) {
        EF_CHECK(batch_solve(c, t, rtol, maxIter, b, x, iters, relres, s));  // warm-up
        EF_CUDA(cudaEventRecord(c->ev[0], s));
        EF_CHECK(batch_solve(c, t, rtol, maxIter, b, x, iters, relres, s));
        EF_CUDA(cudaEventRecord(c->ev[1], s));
        EF_CUDA(cudaEventSynchronize(c->ev[1]));
        float ms = 0.f;
        EF_CUDA(cudaEventElapsedTime(&ms, c->ev[0], c->ev[1]));
        if (msOut) msOut[t] = ms;
        if (ms < best) {
            best = ms;
            bestT = t;
        }
    }
    c->batchTile = bestT;
    if (tileOut) *tileOut = bestT;
    return EF_OK;
}

ef_status ef_batch_norms(ef_ctx* c, const double* R, const double* F, const double* ddU, double* out, void* stream) {
    EF_REQUIRE_FINALIZED(c);
    if (c->batchN == 0) {
        ef_set_error("ef_batch_norms: call ef_batch_setup first");
        return EF_ERR_STATE;
    }
    if (!R || !F || !out) return EF_ERR_ARG;
    return ef_launch_batch_norms(c->batchN, c->dBatchNodePtr, R, F, ddU, out, (cudaStream_t)stream);
}

