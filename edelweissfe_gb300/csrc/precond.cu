// Preconditioner set-up and application on the host side: the sliced-ELL copy of the fine
// system, the aggregation hierarchy (plain or smoothed prolongators, Galerkin operators, damping
// estimates, coarsest inverse), its refresh for a new system and the multigrid cycle.

#include "amg_sa_pattern.h"
#include "ctx.h"

// ---- aggregation multigrid (host setup, device refresh and V-cycle) -------------------------

// greedy aggregation of a block graph: seeds take their whole (unaggregated) neighbourhood,
// left-over nodes join a neighbouring seed aggregate; nodes coupled to nothing but themselves
// (tied nodes, whose DOFs are eliminated) all share one aggregate, so they coarsen away
static int aggregate(int n, const std::vector<int32_t>& rowPtr, const std::vector<int32_t>& colIdx,
                     std::vector<int32_t>& agg) {
    agg.assign(n, -1);
    int nAgg = 0;
    int iso = -1;
    for (int m = 0; m < n; ++m)
        if (rowPtr[m + 1] - rowPtr[m] <= 1) {
            if (iso < 0) iso = nAgg++;
            agg[m] = iso;
        }
    for (int m = 0; m < n; ++m) {
        if (agg[m] != -1) continue;
        bool free = true;
        for (int k = rowPtr[m]; k < rowPtr[m + 1]; ++k)
            if (agg[colIdx[k]] != -1) {
                free = false;
                break;
            }
        if (!free) continue;
        for (int k = rowPtr[m]; k < rowPtr[m + 1]; ++k) agg[colIdx[k]] = nAgg;
        agg[m] = nAgg++;
    }
    std::vector<int32_t> first = agg;
    for (int m = 0; m < n; ++m) {
        if (agg[m] != -1) continue;
        for (int k = rowPtr[m]; k < rowPtr[m + 1]; ++k)
            if (first[colIdx[k]] != -1) {
                agg[m] = first[colIdx[k]];
                break;
            }
    }
    for (int m = 0; m < n; ++m)
        if (agg[m] == -1) agg[m] = nAgg++;
    return nAgg;
}


// vectors of the FGMRES preconditioner (input, output) and the fine-level work vectors (also
// the FGMRES restart residual), whichever base preconditioner runs
ef_status amg_workspace(ef_ctx* c) {
    ef_status st = EF_OK;
    if (!c->vcIn) c->vcIn = dalloc<float>(c->nDof, &st);
    if (!c->vcOut) c->vcOut = dalloc<float>(c->nDof, &st);
    if (!c->fineX) c->fineX = dalloc<float>(c->nDof, &st);
    if (!c->fineT) c->fineT = dalloc<float>(c->nDof, &st);
    return (c->vcIn && c->vcOut && c->fineX && c->fineT) ? EF_OK : st;
}

// ---- sliced-ELL copy of the fine system (kernels in sell.cu) ---------------------------------

// Layout, decided once: slices of 32 block rows in their natural order; when that pads the slots
// by more than 15 % over the blocks, rows are sorted by length (longest first) within windows of
// 4096 rows and the permutation is kept if it pads less; above 50 % padding after that (or with
// EF_SELL=0, or an FP64 system) the CSR kernels stay in use.
static ef_status sell_build(ef_ctx* c) {
    if (c->sellMode >= 0) return EF_OK;
    c->sellMode = 0;
    if (const char* e = getenv("EF_SELL"))
        if (atoi(e) == 0) return EF_OK;
    auto split = [](const char* e, int dflt) {
        if (!e) return dflt;
        const int k = atoi(e);
        return (k == 1 || k == 2 || k == 4 || k == 8) ? k : dflt;
    };
    c->sellSplit = split(getenv("EF_SELL_SPLIT"), c->sellSplit);
    c->sellSplitProduct = split(getenv("EF_SELL_SPLIT_PRODUCT"), c->sellSplitProduct);
    const int n0 = (int)c->nNodes;
    const std::vector<int32_t>& rp = c->hRowPtr0;
    const std::vector<int32_t>& ci = c->hColIdx0;
    if (c->keFp64 || n0 <= 0 || (int64_t)rp.size() != (int64_t)n0 + 1) return EF_OK;
    auto len = [&](int m) { return rp[m + 1] - rp[m]; };
    auto slots = [&](const std::vector<int32_t>& order) {
        int64_t tot = 0;
        for (int s0 = 0; s0 < n0; s0 += 32) {
            int w = 0;
            for (int r = s0; r < std::min(s0 + 32, n0); ++r) w = std::max(w, len(order.empty() ? r : order[r]));
            tot += 32 * (int64_t)w;
        }
        return tot;
    };
    std::vector<int32_t> perm;
    int64_t nE = slots(perm);
    const double nb = (double)c->nBlocks;
    if (nE > 1.15 * nb) {
        std::vector<int32_t> p(n0);
        for (int m = 0; m < n0; ++m) p[m] = m;
        const int W = 4096;
        for (int w0 = 0; w0 < n0; w0 += W)
            std::stable_sort(p.begin() + w0, p.begin() + std::min(w0 + W, n0),
                             [&](int a, int b) { return len(a) > len(b); });
        const int64_t nE2 = slots(p);
        if (nE2 < nE) {
            nE = nE2;
            perm.swap(p);
        }
    }
    const int nS = (n0 + 31) / 32;
    // Diagonal form: when every block column is its row plus one of at most kSellDiaMax node
    // offsets (a structured mesh numbered along grid lines) and the rows keep their order, every
    // slice gets the same slot columns, one per offset in ascending order, zero blocks where a row
    // lacks that neighbour; each row's blocks are then summed in the same (column) order as in
    // the packed slices.  Taken when it pads no more than 15 % over the blocks.
    constexpr int kSellDiaMax = 32;
    std::vector<int32_t> dia;
    {
        bool ok = perm.empty();
        if (const char* e = getenv("EF_SELL_DIA"))
            if (atoi(e) == 0) ok = false;
        for (int m = 0; ok && m < n0; ++m)
            for (int32_t k = rp[m]; k < rp[m + 1]; ++k) {
                const int32_t d = ci[k] - m;
                auto it = std::lower_bound(dia.begin(), dia.end(), d);
                if (it != dia.end() && *it == d) continue;
                if ((int)dia.size() == kSellDiaMax) {
                    ok = false;
                    break;
                }
                dia.insert(it, d);
            }
        if (ok && (double)32 * nS * dia.size() > 1.15 * nb) ok = false;
        // each row's columns ascending (the slot order must be the row's block order)
        for (int m = 0; ok && m < n0; ++m)
            for (int32_t k = rp[m] + 1; k < rp[m + 1]; ++k)
                if (ci[k] <= ci[k - 1]) ok = false;
        if (!ok) dia.clear();
    }
    if (!dia.empty()) nE = 32 * (int64_t)nS * (int64_t)dia.size();
    if (nE > 1.5 * nb || nE >= ((int64_t)1 << 31) / 9) return EF_OK;
    std::vector<int64_t> off(nS + 1, 0);
    std::vector<int32_t> col(nE), src(nE);
    if (!dia.empty()) {
        const int W = (int)dia.size();
        for (int s = 0; s < nS; ++s) {
            off[s + 1] = off[s] + 32 * (int64_t)W;
            for (int i = 0; i < 32; ++i) {
                const int r = 32 * s + i;
                int32_t k = r < n0 ? rp[r] : 0;
                for (int j = 0; j < W; ++j) {
                    const int64_t t = off[s] + 32 * (int64_t)j + i;
                    const int64_t cc = (int64_t)r + dia[j];
                    col[t] = (int32_t)std::min<int64_t>(std::max<int64_t>(cc, 0), n0 - 1);
                    if (r < n0 && k < rp[r + 1] && ci[k] == cc) {
                        src[t] = k++;
                    } else {
                        src[t] = -1;
                    }
                }
                if (r < n0 && k != rp[r + 1]) {
                    ef_set_error("sliced-ELL diagonal form: a row's blocks do not follow the offsets");
                    return EF_ERR_STATE;
                }
            }
        }
    }
    for (int s = 0; dia.empty() && s < nS; ++s) {
        int w = 0;
        for (int r = 32 * s; r < std::min(32 * s + 32, n0); ++r) w = std::max(w, len(perm.empty() ? r : perm[r]));
        off[s + 1] = off[s] + 32 * (int64_t)w;
        for (int j = 0; j < w; ++j)
            for (int i = 0; i < 32; ++i) {
                const int r = 32 * s + i;
                const int64_t t = off[s] + 32 * (int64_t)j + i;
                if (r < n0) {
                    const int m = perm.empty() ? r : perm[r];
                    const bool real = j < len(m);
                    src[t] = real ? rp[m] + j : -1;
                    col[t] = real ? ci[rp[m] + j] : m;
                } else {
                    src[t] = -1;
                    col[t] = n0 - 1;
                }
            }
    }
    ef_status st = EF_OK;
    EF_CHECK(upload(&c->dSellOff, off));
    EF_CHECK(upload(&c->dSellCol, col));
    EF_CHECK(upload(&c->dSellSrc, src));
    if (!perm.empty()) EF_CHECK(upload(&c->dSellPerm, perm));
    if (!dia.empty()) {
        EF_CHECK(upload(&c->dSellDia, dia));
        c->sellDiaN = (int)dia.size();
    }
    c->dSellV9 = dalloc<float>(9 * (size_t)nE, &st);
    if (!c->dSellV9) return st;
    if (c->amgBf16) {
        c->dSellV8 = dalloc<uint4>((size_t)nE, &st);
        c->dSellV1 = dalloc<uint16_t>((size_t)nE, &st);
        if (!c->dSellV8 || !c->dSellV1) return st;
    }
    c->sellSlices = nS;
    c->sellE = nE;
    c->sellMode = 1;
    c->sellStale = true;
    return EF_OK;
}

// the SELL values from the assembled FP32 blocks (after every assembly)
ef_status sell_refresh(ef_ctx* c, cudaStream_t s) {
    EF_CHECK(sell_build(c));
    if (c->sellMode != 1 || !c->sellStale) return EF_OK;
    EF_CHECK(ef_launch_sell_refresh(c->sellE, c->dSellSrc, (const float*)c->dBsrVals, c->dSellV9, c->dSellV8,
                                    c->dSellV1, c->dSellCol, c->sellScaled ? (const float*)c->dBinv : nullptr,
                                    c->dMask, s));
    c->sellStale = false;
    return EF_OK;
}

ef_status amg_build(ef_ctx* c) {
    if (!c->amg.empty()) return EF_OK;
    if (const char* e = getenv("EF_AMG_SMOOTHED")) c->amgSmoothed = atoi(e) != 0;
    if (const char* e = getenv("EF_SA_TWOSTAGE")) c->saTransfer = atoi(e) != 0 ? 1 : 0;
    if (const char* e = getenv("EF_SA_TRANSFER")) c->saTransfer = std::min(2, std::max(0, atoi(e)));
    if (const char* e = getenv("EF_AMG_FUSED_POST")) c->postFused = atoi(e) != 0;
    // smoothed prolongators: one sweep before and after, V-cycle (the fastest cfg 2 load step of
    // 1/1, 2/2 x V, W on level 1); plain aggregation: two sweeps and a W-cycle on level 1
    if (c->amgSmoothed) {
        c->amgSweeps = 1;
        c->amgWLevels = 0;
    }
    if (const char* e = getenv("EF_AMG_OMEGA")) c->amgOmega = (float)atof(e);
    if (const char* e = getenv("EF_AMG_SWEEPS")) c->amgSweeps = std::max(1, atoi(e));
    c->amgPre = c->amgPost = c->amgSweeps;
    if (const char* e = getenv("EF_AMG_PRE")) c->amgPre = std::max(0, atoi(e));  // 0: no pre-smoothing
    if (const char* e = getenv("EF_AMG_POST")) c->amgPost = std::max(0, atoi(e));  // 0: no post-smoothing
    if (const char* e = getenv("EF_AMG_WLEVELS")) c->amgWLevels = std::max(0, atoi(e));
    c->amgPreC = c->amgPre;
    c->amgPostC = c->amgPost;
    if (const char* e = getenv("EF_AMG_PRE_COARSE")) c->amgPreC = std::max(0, atoi(e));
    if (const char* e = getenv("EF_AMG_POST_COARSE")) c->amgPostC = std::max(0, atoi(e));
    if (const char* e = getenv("EF_AMG_ALPHA")) c->amgAlpha = (float)atof(e);
    if (const char* e = getenv("EF_AMG_CYCLE")) c->amgCycle = std::max(1, atoi(e));
    if (const char* e = getenv("EF_AMG_BF16")) c->amgBf16 = atoi(e) != 0;
    if (const char* e = getenv("EF_AMG_SMOOTHER")) c->amgCheb = strcmp(e, "cheb") == 0;
    if (const char* e = getenv("EF_AMG_CLUSTER")) c->amgCluster = atoi(e) != 0;
    if (const char* e = getenv("EF_AMG_BF16_COARSE")) c->amgBf16Coarse = atoi(e) != 0;
    if (c->amgSmoothed && !getenv("EF_AMG_ALPHA")) c->amgAlpha = 1.0f;  // smoothed prolongators need no over-correction
    ef_status st = EF_OK;
    const int n0 = (int)c->nNodes;
    const int BCo = ef_amg_coarse_dofs();
    // fine block -> block row
    std::vector<int32_t> rob0(c->nBlocks);
    for (int m = 0; m < n0; ++m)
        for (int k = c->hRowPtr0[m]; k < c->hRowPtr0[m + 1]; ++k) rob0[k] = m;
    EF_CHECK(upload(&c->dRowOfBlock0, rob0));
    EF_CHECK(amg_workspace(c));
    EF_CHECK(sell_build(c));
    if (c->amgBf16 && c->sellMode != 1) {  // (with the SELL copy the fine level reads its BF16 values)
        c->dBsrValsH = dalloc<uint16_t>((size_t)c->nBlocks * 9 + 32, &st);  // 16-byte words + 1 value per block (+ padding)
        if (!c->dBsrValsH) return st;
        bool staged = false;  // measured slower than the unstaged kernel (EF_AMG_STAGED=1 turns it on)
        if (const char* e = getenv("EF_AMG_STAGED")) staged = atoi(e) != 0;
        c->stageCap = staged ? ef_stage_cap(n0, c->hRowPtr0.data()) : 0;
        if (c->stageCap > 4096) c->stageCap = 0;  // rows too long for a shared-memory stage: unstaged kernel
    }
    const std::vector<int32_t>* pRow = &c->hRowPtr0;
    const std::vector<int32_t>* pCol = &c->hColIdx0;
    std::vector<double> finePos(3 * (size_t)n0);
    for (int m = 0; m < n0; ++m)
        for (int k = 0; k < 3; ++k) finePos[3 * m + k] = c->hX[3 * m + k];
    const std::vector<double>* pPos = &finePos;
    int nFine = n0;
    while (nFine > ef_max_coarsest_nodes()) {
        AmgLevel L;
        // frees the level's device arrays on an early error return, until the context owns them
        struct Guard {
            AmgLevel* L;
            ~Guard() {
                if (L) L->free_device();
            }
        } guard{&L};
        const int nC = aggregate(nFine, *pRow, *pCol, L.hAgg);
        if (nC >= nFine) break;  // no coarsening progress
        L.nN = nC;
        // members of each coarse node (increasing finer index), centroids and offsets
        L.hAggPtr.assign(nC + 1, 0);
        for (int m = 0; m < nFine; ++m) L.hAggPtr[L.hAgg[m] + 1]++;
        for (int I = 0; I < nC; ++I) L.hAggPtr[I + 1] += L.hAggPtr[I];
        L.hAggIdx.resize(nFine);
        {
            std::vector<int32_t> fill(L.hAggPtr.begin(), L.hAggPtr.end() - 1);
            for (int m = 0; m < nFine; ++m) L.hAggIdx[fill[L.hAgg[m]]++] = m;
        }
        L.hCentroid.assign(3 * (size_t)nC, 0.0);
        for (int m = 0; m < nFine; ++m)
            for (int k = 0; k < 3; ++k) L.hCentroid[3 * L.hAgg[m] + k] += (*pPos)[3 * m + k];
        for (int I = 0; I < nC; ++I) {
            const double cnt = (double)(L.hAggPtr[I + 1] - L.hAggPtr[I]);
            for (int k = 0; k < 3; ++k) L.hCentroid[3 * I + k] /= cnt;
        }
        L.hOffs.resize(3 * (size_t)nFine);
        for (int m = 0; m < nFine; ++m)
            for (int k = 0; k < 3; ++k) L.hOffs[3 * m + k] = (float)((*pPos)[3 * m + k] - L.hCentroid[3 * L.hAgg[m] + k]);
        // coarse pattern: aggregate adjacency, or with smoothed prolongators the pattern of P^T A P
        // (a superset)
        std::vector<std::vector<int32_t>> cols(nC);
        SAPattern SA;
        if (c->amgSmoothed) {
            build_sa_pattern(nFine, pRow->data(), pCol->data(), L.hAgg.data(), nC, SA);
            for (int I = 0; I < nC; ++I) cols[I].assign(SA.cCol.begin() + SA.cRowPtr[I], SA.cCol.begin() + SA.cRowPtr[I + 1]);
        } else {
            for (int m = 0; m < nFine; ++m)
                for (int k = (*pRow)[m]; k < (*pRow)[m + 1]; ++k) cols[L.hAgg[m]].push_back(L.hAgg[(*pCol)[k]]);
        }
        L.hRowPtr.assign(nC + 1, 0);
        for (int I = 0; I < nC; ++I) {
            auto& v = cols[I];
            std::sort(v.begin(), v.end());
            v.erase(std::unique(v.begin(), v.end()), v.end());
            L.hRowPtr[I + 1] = L.hRowPtr[I] + (int32_t)v.size();
        }
        L.nBlocks = L.hRowPtr[nC];
        L.hColIdx.resize(L.nBlocks);
        std::vector<int32_t> rob(L.nBlocks);
        std::vector<int64_t> diag(nC, -1);
        for (int I = 0; I < nC; ++I)
            for (size_t j = 0; j < cols[I].size(); ++j) {
                const int64_t k = L.hRowPtr[I] + (int64_t)j;
                L.hColIdx[k] = cols[I][j];
                rob[k] = I;
                if (cols[I][j] == I) diag[I] = k;
            }
        // Galerkin map: finer blocks in increasing order, grouped by their coarse block
        const int64_t nFineBlocks = (*pRow)[nFine];
        std::vector<int64_t> gcount(L.nBlocks + 1, 0);
        std::vector<int32_t> target(nFineBlocks);
        for (int m = 0; m < nFine; ++m) {
            const int I = L.hAgg[m];
            for (int k = (*pRow)[m]; k < (*pRow)[m + 1]; ++k) {
                const int J = L.hAgg[(*pCol)[k]];
                const int32_t* b = L.hColIdx.data() + L.hRowPtr[I];
                const int32_t* e = L.hColIdx.data() + L.hRowPtr[I + 1];
                const int64_t S = L.hRowPtr[I] + (std::lower_bound(b, e, J) - b);
                target[k] = (int32_t)S;
                gcount[S + 1]++;
            }
        }
        for (int64_t S = 0; S < L.nBlocks; ++S) gcount[S + 1] += gcount[S];
        std::vector<int32_t> gsrc(nFineBlocks);
        {
            std::vector<int64_t> fill(gcount.begin(), gcount.end() - 1);
            for (int64_t f = 0; f < nFineBlocks; ++f) gsrc[fill[target[f]]++] = (int32_t)f;
        }
        EF_CHECK(upload(&L.rowPtr, L.hRowPtr));
        EF_CHECK(upload(&L.colIdx, L.hColIdx));
        EF_CHECK(upload(&L.rowOfBlock, rob));
        EF_CHECK(upload(&L.diagPos, diag));
        EF_CHECK(upload(&L.agg, L.hAgg));
        EF_CHECK(upload(&L.offs, L.hOffs));
        EF_CHECK(upload(&L.aggPtr, L.hAggPtr));
        EF_CHECK(upload(&L.aggIdx, L.hAggIdx));
        EF_CHECK(upload(&L.gseg, gcount));
        EF_CHECK(upload(&L.gsrc, gsrc));
        if (c->amgSmoothed) {
            L.saNP = (int64_t)SA.pCol.size();
            L.saNAP = (int64_t)SA.apCol.size();
            std::vector<int32_t> apRow(L.saNAP);
            for (int m = 0; m < nFine; ++m)
                for (int32_t a = SA.apRowPtr[m]; a < SA.apRowPtr[m + 1]; ++a) apRow[a] = m;
            EF_CHECK(upload(&L.saPRowPtr, SA.pRowPtr));
            EF_CHECK(upload(&L.saPCol, SA.pCol));
            EF_CHECK(upload(&L.saPRow, SA.pRow));
            EF_CHECK(upload(&L.saPSeg, SA.pSeg));
            EF_CHECK(upload(&L.saPSrc, SA.pSrc));
            EF_CHECK(upload(&L.saTPtr, SA.tPtr));
            EF_CHECK(upload(&L.saTIdx, SA.tIdx));
            EF_CHECK(upload(&L.saApRow, apRow));
            EF_CHECK(upload(&L.saApSeg, SA.apSeg));
            EF_CHECK(upload(&L.saApK, SA.apK));
            EF_CHECK(upload(&L.saApP, SA.apP));
            EF_CHECK(upload(&L.saCSeg, SA.cSeg));
            EF_CHECK(upload(&L.saCP, SA.cP));
            EF_CHECK(upload(&L.saCAP, SA.cAP));
            const int bfL = c->amg.empty() ? 3 : BCo;
            L.saPv = dalloc<float>((size_t)std::max<int64_t>(1, L.saNP) * bfL * BCo, &st);
            L.saAPv = dalloc<float>((size_t)std::max<int64_t>(1, L.saNAP) * bfL * BCo, &st);
            L.saW = dalloc<float>(1, &st);
            L.saC = dalloc<float>((size_t)std::max<int64_t>(1, L.saNP) * BCo, &st);
            if (!L.saPv || !L.saAPv || !L.saW || !L.saC) return st;
            {
                // AP by groups of finer rows where their pair products fit the shared memory
                const int G = ef_sa_ap_rows();
                int64_t cap = 0;
                for (int r0 = 0; r0 < nFine; r0 += G)
                    cap = std::max(cap, SA.apSeg[SA.apRowPtr[std::min(r0 + G, nFine)]] - SA.apSeg[SA.apRowPtr[r0]]);
                if (cap > 0 && ef_sa_ap_rows_smem(bfL, (int)std::min<int64_t>(cap, 1 << 20)) <= 48 * 1024) {
                    EF_CHECK(upload(&L.saApRowPtr, SA.apRowPtr));
                    L.saApCap = (int)cap;
                }
            }
            if (c->amg.empty() && c->postFused && c->sellMode == 1 && L.saNAP > 0) {
                // fused fine-level post-smoothing: C in the pattern of AP, sliced over the fine rows
                // (slices of 32 rows, column-major slots; rows sorted by length within windows of
                // 4096, as the A P rows run from 1 to 27 blocks), and for each AP block its P block
                const int nS = (nFine + 31) / 32;
                auto apLen = [&](int m) { return SA.apRowPtr[m + 1] - SA.apRowPtr[m]; };
                std::vector<int32_t> pperm(nFine);
                for (int m = 0; m < nFine; ++m) pperm[m] = m;
                for (int w0 = 0; w0 < nFine; w0 += 4096)
                    std::stable_sort(pperm.begin() + w0, pperm.begin() + std::min(w0 + 4096, nFine),
                                     [&](int a, int b) { return apLen(a) > apLen(b); });
                std::vector<int64_t> poff(nS + 1, 0);
                for (int sl = 0; sl < nS; ++sl) {
                    int w = 0;
                    for (int r = 32 * sl; r < std::min(32 * sl + 32, nFine); ++r) w = std::max(w, apLen(pperm[r]));
                    poff[sl + 1] = poff[sl] + 32 * (int64_t)w;
                }
                const int64_t nSlot = poff[nS];
                std::vector<int32_t> pcol(nSlot, 0), psrc(nSlot, -1), apToP(L.saNAP, -1);
                for (int sl = 0; sl < nS; ++sl) {
                    const int w = (int)((poff[sl + 1] - poff[sl]) / 32);
                    for (int i = 0; i < 32; ++i) {
                        if (32 * sl + i >= nFine) continue;
                        const int m = pperm[32 * sl + i];
                        for (int j = 0; j < w; ++j) {
                            const int64_t a = SA.apRowPtr[m] + j;
                            if (a >= SA.apRowPtr[m + 1]) break;
                            const int64_t t = poff[sl] + 32 * (int64_t)j + i;
                            pcol[t] = SA.apCol[a];
                            psrc[t] = (int32_t)a;
                        }
                    }
                }
                for (int m = 0; m < nFine; ++m)
                    for (int32_t a = SA.apRowPtr[m]; a < SA.apRowPtr[m + 1]; ++a)
                        apToP[a] = (int32_t)sa_find(SA.pCol, SA.pRowPtr[m], SA.pRowPtr[m + 1], SA.apCol[a]);
                EF_CHECK(upload(&c->dPostOff, poff));
                EF_CHECK(upload(&c->dPostPerm, pperm));
                EF_CHECK(upload(&c->dPostCol, pcol));
                EF_CHECK(upload(&c->dPostSrc, psrc));
                EF_CHECK(upload(&c->dPostApToP, apToP));
                c->dPostQ0 = dalloc<uint4>((size_t)nSlot, &st);
                c->dPostQ1 = dalloc<uint4>((size_t)nSlot, &st);
                c->dPostQ2 = dalloc<uint32_t>((size_t)nSlot, &st);
                if (!c->dPostQ0 || !c->dPostQ1 || !c->dPostQ2) return st;
                c->postSlices = nS;
                c->postSlots = nSlot;
            }
            if (!c->amg.empty() && c->postFused && L.saNAP > 0) {
                // fused post-smoothing of this 6-DOF finer level
                std::vector<int32_t> apToP(L.saNAP, -1);
                for (int m = 0; m < nFine; ++m)
                    for (int32_t a = SA.apRowPtr[m]; a < SA.apRowPtr[m + 1]; ++a)
                        apToP[a] = (int32_t)sa_find(SA.pCol, SA.pRowPtr[m], SA.pRowPtr[m + 1], SA.apCol[a]);
                EF_CHECK(upload(&L.postRowPtr, SA.apRowPtr));
                EF_CHECK(upload(&L.postCol, SA.apCol));
                EF_CHECK(upload(&L.postApToP, apToP));
                L.postC = dalloc<float>((size_t)L.saNAP * BCo * BCo, &st);
                if (!L.postC) return st;
            }
            if (c->saTransfer == 2 && L.saNP > 0) {
                // one-pass transfers where the prolongation's block products of a group of
                // consecutive finer rows fit the shared memory
                const int G = ef_sa_prolong_onepass_rows();
                int cap = 0;
                for (int r0 = 0; r0 < nFine; r0 += G)
                    cap = std::max(cap, SA.pRowPtr[std::min(r0 + G, nFine)] - SA.pRowPtr[r0]);
                if (ef_sa_prolong_onepass_smem(bfL, cap) <= 48 * 1024) {
                    std::vector<int32_t> rowT(L.saNP);
                    for (int64_t k = 0; k < L.saNP; ++k) rowT[k] = SA.pRow[SA.tIdx[k]];
                    EF_CHECK(upload(&L.saRowT, rowT));
                    bool h = bfL == 3;
                    if (const char* e = getenv("EF_SA_PT_BF16")) h = h && atoi(e) != 0;
                    if (h) {  // BF16 copy for the fine restriction
                        L.saPTh0 = dalloc<uint4>((size_t)L.saNP, &st);
                        L.saPTh1 = dalloc<uint4>((size_t)L.saNP, &st);
                        L.saPTh2 = dalloc<uint32_t>((size_t)L.saNP, &st);
                        if (!L.saPTh0 || !L.saPTh1 || !L.saPTh2) return st;
                    } else {
                        L.saPT = dalloc<float>((size_t)L.saNP * bfL * BCo, &st);
                        if (!L.saPT) return st;
                    }
                    L.saCap = cap;
                    L.saOnePass = true;
                }
            }
        }
        L.vals = dalloc<float>((size_t)L.nBlocks * BCo * BCo, &st);
        L.binv = dalloc<float>((size_t)nC * BCo * BCo, &st);
        L.dead = dalloc<uint8_t>((size_t)BCo * nC, &st);
        L.x = dalloc<float>((size_t)BCo * nC, &st);
        L.r = dalloc<float>((size_t)BCo * nC, &st);
        L.t = dalloc<float>((size_t)BCo * nC, &st);
        L.x2 = dalloc<float>((size_t)BCo * nC, &st);
        if (!L.vals || !L.binv || !L.dead || !L.x || !L.r || !L.t || !L.x2) return st;
        if (c->amgBf16Coarse) {
            L.valsH = dalloc<uint16_t>((size_t)L.nBlocks * BCo * BCo, &st);
            if (!L.valsH) return st;
        }
        guard.L = nullptr;
        c->amg.push_back(std::move(L));
        pRow = &c->amg.back().hRowPtr;
        pCol = &c->amg.back().hColIdx;
        pPos = &c->amg.back().hCentroid;
        nFine = nC;
    }
    c->chebD.assign(c->amg.size(), nullptr);  // Chebyshev directions of the smoothed levels
    for (size_t l = 0; l < c->amg.size(); ++l) {
        const size_t nl = l == 0 ? (size_t)c->nDof : (size_t)BCo * c->amg[l - 1].nN;
        c->chebD[l] = dalloc<float>(nl, &st);
        if (!c->chebD[l]) return st;
    }
    if (c->amg.empty() || c->amg.back().nN > ef_max_coarsest_nodes()) {
        ef_set_error("multigrid: the block graph does not coarsen to a dense-solvable size");
        return EF_ERR_ARG;
    }
    const int nc = BCo * c->amg.back().nN;
    c->amgCoarsestInv = dalloc<float>((size_t)nc * nc, &st);
    if (!c->amgCoarsestInv) return st;
    // fused cycles without a pre-sweep launch: the fine BF16 copy scaled to K (M D^-1), and
    // B = A (M D^-1) beside each 6-DOF level whose cycle is fused (EF_AMG_SCALED=0: keep the sweep)
    bool scaled = true;
    if (const char* e = getenv("EF_AMG_SCALED")) scaled = atoi(e) != 0;
    const bool oneOne = c->amgPre == 1 && c->amgPost == 1 && !c->amgCheb && c->amgSmoothed;
    c->sellScaled = scaled && oneOne && c->postSlots > 0 && c->amgBf16 && c->sellMode == 1;
    c->sellStale = true;
    if (scaled && c->amgPreC == 1 && c->amgPostC == 1 && !c->amgCheb && c->amgSmoothed)
        for (size_t k = 0; k + 1 < c->amg.size(); ++k)
            if (c->amg[k + 1].postC) {
                c->amg[k].valsB = dalloc<float>((size_t)c->amg[k].nBlocks * BCo * BCo, &st);
                if (!c->amg[k].valsB) return st;
            }
    EF_CHECK(amg_workspace(c));
    c->amgStale = true;
    return EF_OK;
}

ef_status amg_vcycle(ef_ctx* c, int l, const float* r, float* x, cudaStream_t s);

// capture the preconditioner application (fixed device pointers; values may change later)
// Phase program of the cycle at level l >= 1 (6-DOF nodes) from right-hand side r into x: the
// same operations, order and buffers as amg_vcycle's block-Jacobi path.
static void amg_cycle_ops(const ef_ctx* c, int l, const float* r, float* x, std::vector<ef::CoarseOp>& ops) {
    const int nL = (int)c->amg.size();
    const int BCo = ef_amg_coarse_dofs();
    auto op = [](int type, int n) {
        ef::CoarseOp o{};
        o.type = type;
        o.n = n;
        return o;
    };
    if (l == nL) {
        const AmgLevel& C = c->amg.back();
        ef::CoarseOp o = op(ef::COP_COARSEST, BCo * C.nN);
        o.f0 = c->amgCoarsestInv;
        o.in = r;
        o.mask = C.dead;
        o.out = x;
        ops.push_back(o);
        return;
    }
    const AmgLevel& L = c->amg[l - 1];
    const AmgLevel& Cn = c->amg[l];
    const float omega = l < (int)c->levelOmega.size() ? c->levelOmega[l] : c->amgOmega;
    auto sweep = [&](const float* xin, float* xout) {
        ef::CoarseOp o = op(ef::COP_SWEEP, L.nN);
        o.p0 = L.rowPtr;
        o.p1 = L.colIdx;
        o.f0 = L.vals;
        o.f1 = L.binv;
        o.mask = L.dead;
        o.in = xin;
        o.rhs = r;
        o.out = xout;
        o.omega = omega;
        ops.push_back(o);
    };
    float* x2 = L.x2;
    float* cur = ((c->amgPreC + c->amgPostC) & 1) ? x : x2;
    {
        ef::CoarseOp o = op(ef::COP_BJ, L.nN);
        o.f1 = L.binv;
        o.mask = L.dead;
        o.in = r;
        o.out = cur;
        o.omega = omega;
        ops.push_back(o);
    }
    for (int k = 1; k < c->amgPreC; ++k) {
        float* nxt = cur == x ? x2 : x;
        sweep(cur, nxt);
        cur = nxt;
    }
    const int reps = (c->amgCycle > 1 && l <= c->amgWLevels) ? c->amgCycle : 1;
    for (int rep = 0; rep < reps; ++rep) {
        ef::CoarseOp o = op(ef::COP_RESID, L.nN);
        o.p0 = L.rowPtr;
        o.p1 = L.colIdx;
        o.f0 = L.vals;
        o.mask = L.dead;
        o.in = cur;
        o.rhs = r;
        o.out = L.t;
        ops.push_back(o);
        ef::CoarseOp rs = op(ef::COP_RESTRICT, Cn.nN);
        rs.p0 = Cn.aggPtr;
        rs.p1 = Cn.aggIdx;
        rs.f0 = Cn.offs;
        rs.mask = Cn.dead;
        rs.in = L.t;
        rs.out = Cn.r;
        ops.push_back(rs);
        amg_cycle_ops(c, l + 1, Cn.r, Cn.x, ops);
        ef::CoarseOp pr = op(ef::COP_PROLONG, L.nN);
        pr.p0 = Cn.agg;
        pr.f0 = Cn.offs;
        pr.mask = L.dead;
        pr.in = Cn.x;
        pr.out = cur;
        pr.omega = c->amgAlpha;
        ops.push_back(pr);
    }
    for (int k = 0; k < c->amgPostC; ++k) {
        float* nxt = cur == x ? x2 : x;
        sweep(cur, nxt);
        cur = nxt;
    }
}

// Chooses the level whose coarse correction (restriction, the whole cycle below, prolongation)
// runs as one coarse_cycle_kernel launch: the first level >= 1 whose next coarser level has at
// most kClusterMaxNodes nodes; builds and uploads its phase program (before a graph capture).
static ef_status amg_prepare_cluster(ef_ctx* c) {
    constexpr int kClusterMaxNodes = 2048;
    c->clusterLevel = -1;
    c->nCoarseOps = 0;
    const int nL = (int)c->amg.size();
    if (!c->amgCluster || c->amgCheb || c->amgSmoothed || c->amgPreC < 1 || c->amgPostC < 1) return EF_OK;
    int lc = -1;
    for (int l = 1; l < nL; ++l)
        if (c->amg[l].nN <= kClusterMaxNodes) {
            lc = l;
            break;
        }
    if (lc < 0) return EF_OK;
    const AmgLevel& L = c->amg[lc - 1];
    const AmgLevel& Cn = c->amg[lc];
    // level lc's iterate at its coarse correction: amg_vcycle's buffer alternation of the
    // pre-smoothing replayed (level lc's output vector is L.x, its second vector L.x2)
    float* x = L.x;
    float* cur = ((c->amgPreC + c->amgPostC) & 1) ? x : L.x2;
    for (int k = 1; k < c->amgPreC; ++k) cur = cur == x ? L.x2 : x;
    std::vector<ef::CoarseOp> ops;
    ef::CoarseOp rs{};
    rs.type = ef::COP_RESTRICT;
    rs.n = Cn.nN;
    rs.p0 = Cn.aggPtr;
    rs.p1 = Cn.aggIdx;
    rs.f0 = Cn.offs;
    rs.mask = Cn.dead;
    rs.in = L.t;
    rs.out = Cn.r;
    ops.push_back(rs);
    amg_cycle_ops(c, lc + 1, Cn.r, Cn.x, ops);
    ef::CoarseOp pr{};
    pr.type = ef::COP_PROLONG;
    pr.n = L.nN;
    pr.p0 = Cn.agg;
    pr.f0 = Cn.offs;
    pr.mask = L.dead;
    pr.in = Cn.x;
    pr.out = cur;
    pr.omega = c->amgAlpha;
    ops.push_back(pr);
    if (!c->dCoarseOps || (int)ops.size() > c->nCoarseOpsCap) {
        if (c->dCoarseOps) cudaFree(c->dCoarseOps);
        c->dCoarseOps = nullptr;
        ef_status st = EF_OK;
        c->dCoarseOps = dalloc<ef::CoarseOp>(ops.size(), &st);
        if (!c->dCoarseOps) return st;
        c->nCoarseOpsCap = (int)ops.size();
    }
    EF_CUDA(cudaMemcpy(c->dCoarseOps, ops.data(), sizeof(ef::CoarseOp) * ops.size(), cudaMemcpyHostToDevice));
    c->nCoarseOps = (int)ops.size();
    c->clusterLevel = lc;
    c->clusterCur = cur;
    return EF_OK;
}

ef_status amg_capture(ef_ctx* c) {
    if (c->vcGraph) return EF_OK;
    EF_CHECK(amg_prepare_cluster(c));
    if (!c->capStream) EF_CUDA(cudaStreamCreateWithFlags(&c->capStream, cudaStreamNonBlocking));
    EF_CUDA(cudaStreamBeginCapture(c->capStream, cudaStreamCaptureModeThreadLocal));
    long long captured = 0;
    t_captureCount = &captured;
    const ef_status st = amg_vcycle(c, 0, c->vcIn, c->vcOut, c->capStream);
    t_captureCount = nullptr;
    c->vcGraphKernels = captured;
    cudaGraph_t g = nullptr;
    const cudaError_t e = cudaStreamEndCapture(c->capStream, &g);
    if (st != EF_OK) return st;
    if (e != cudaSuccess) {
        ef_set_error(std::string("V-cycle capture: ") + cudaGetErrorString(e));
        return EF_ERR_CUDA;
    }
    EF_CUDA(cudaGraphInstantiate(&c->vcGraph, g, 0));
    cudaGraphDestroy(g);
    return EF_OK;
}

// A coarse DOF (translation or rotation of an aggregate) is dead when its prolongation column
// vanishes on every live finer DOF (all members clamped, or a rotation about an axis through
// all free members).
static void amg_dead_mask(const AmgLevel& L, int bf, const uint8_t* fineDead, std::vector<uint8_t>& dead) {
    const int BCo = ef_amg_coarse_dofs();
    dead.assign((size_t)BCo * L.nN, 1);
    for (int I = 0; I < L.nN; ++I) {
        double colNorm[6] = {0, 0, 0, 0, 0, 0};
        double scale = 0.0;
        for (int k = L.hAggPtr[I]; k < L.hAggPtr[I + 1]; ++k) {
            const int m = L.hAggIdx[k];
            const double dx = L.hOffs[3 * m], dy = L.hOffs[3 * m + 1], dz = L.hOffs[3 * m + 2];
            scale = std::max(scale, dx * dx + dy * dy + dz * dz);
            // rows of P_m (bf x 6)
            double P[6][6] = {};
            P[0][0] = P[1][1] = P[2][2] = 1.0;
            P[1][3] = -dz;
            P[2][3] = dy;
            P[0][4] = dz;
            P[2][4] = -dx;
            P[0][5] = -dy;
            P[1][5] = dx;
            if (bf == 6) P[3][3] = P[4][4] = P[5][5] = 1.0;
            for (int i = 0; i < bf; ++i) {
                if (fineDead[(size_t)bf * m + i]) continue;
                for (int j = 0; j < 6; ++j) colNorm[j] += P[i][j] * P[i][j];
            }
        }
        const double tol = 1e-12 * std::max(scale, 1e-300);
        for (int j = 0; j < 3; ++j) dead[BCo * I + j] = colNorm[j] > 0.5 ? 0 : 1;
        for (int j = 3; j < 6; ++j) dead[BCo * I + j] = colNorm[j] > tol && scale > 0.0 ? 0 : 1;
    }
}

// Damping of the block-Jacobi smoother on every smoothed level.  lambda, the largest eigenvalue of
// D^-1 A, is estimated by 12 power iterations from a fixed pseudo-random vector; damped Jacobi
// smoothing is stable for omega lambda < 2.  Where amgOmega lambda exceeds 1.85 (quadratic
// elements raise lambda well above its hex8 value of about 2) the level uses 4 / (3 lambda),
// quantised to 1/64 so that small changes keep the captured cycle; any change re-captures it.
static constexpr int kPowerSteps = 13;  // power-iteration steps per level

// scratch of the damping estimate (allocated once)
static ef_status amg_power_alloc(ef_ctx* c) {
    ef_status st = EF_OK;
    if (!c->amgPow[0]) {
        c->amgPow[0] = dalloc<float>(c->nDof, &st);
        c->amgPow[1] = dalloc<float>(c->nDof, &st);
        c->amgZero = dalloc<float>(c->nDof, &st);
        c->amgPowFac = dalloc<float>(1, &st);
        if (st != EF_OK) return st;
        EF_CUDA(cudaMemset(c->amgZero, 0, sizeof(float) * c->nDof));
    }
    if (!c->nnRed) {  // reduction scratch shared with the learned correction
        c->nnPartN = 2 * c->nSM;
        c->nnRed = dalloc<double>(3 * (size_t)c->nnPartN + 8, &st);
        if (!c->nnRed) return st;
    }
    const int nL = (int)c->amg.size();
    if (!c->amgNorms || c->amgNormsCap < 3 * kPowerSteps * nL) {
        if (c->amgNorms) cudaFree(c->amgNorms);
        c->amgNorms = dalloc<double>((size_t)3 * kPowerSteps * nL, &st);
        if (!c->amgNorms) return st;
        c->amgNormsCap = 3 * kPowerSteps * nL;
    }
    return EF_OK;
}

// lambda_max(D^-1 A) of level l by power iteration, entirely on the device (normalised by the
// device-side norm); the last step's squared norm, lambda^2, is left at
// amgNorms[3 (l kPowerSteps + kPowerSteps - 1)]
static ef_status amg_power(ef_ctx* c, int l, cudaStream_t s) {
    const int BCo = ef_amg_coarse_dofs();
    const bool fine = l == 0;
    const int bs = fine ? 3 : BCo;
    const int nN = fine ? (int)c->nNodes : c->amg[l - 1].nN;
    const int32_t* rowPtr = fine ? c->dRowPtr : c->amg[l - 1].rowPtr;
    const int32_t* colIdx = fine ? c->dColIdx : c->amg[l - 1].colIdx;
    const float* vals = fine ? (const float*)c->dBsrVals : c->amg[l - 1].vals;
    const float* binv = fine ? (const float*)c->dBinv : c->amg[l - 1].binv;
    const uint8_t* mask = fine ? c->dMask : c->amg[l - 1].dead;
    const int64_t n = (int64_t)bs * nN;
    float* a = c->amgPow[0];
    float* b = c->amgPow[1];
    // the fine level through the sliced-ELL product, which scales its input by 1 / |a| and applies
    // the block inverses in its epilogue: b = D^-1 K (a / |a|), one launch per step
    const bool sellStep = fine && c->sellMode == 1 && !c->sellStale;
    EF_CHECK(ef_launch_fill_hash(n, a, s));
    for (int it = 0; it < kPowerSteps; ++it) {
        double* n2 = c->amgNorms + 3 * (l * kPowerSteps + it);
        EF_CHECK(ef_mpnn_sumsq(n, 1, a, nullptr, mask, c->nnRed, c->nnPartN, n2, s, c->amgPowFac));
        if (it + 1 == kPowerSteps) break;
        if (sellStep) {
            EF_CHECK(ef_launch_sell_spmv3(nN, c->sellSlices, c->dSellOff, c->dSellPerm, c->dSellCol, c->dSellV9, a,
                                          mask, b, nullptr, c->sellSplitProduct, s, c->amgPowFac, c->dSellDia,
                                          binv));
            std::swap(a, b);
            continue;
        }
        EF_CHECK(ef_launch_scale_by(n, a, c->amgPowFac, s));
        EF_CHECK(ef_launch_level_residual(bs, nN, rowPtr, colIdx, vals, a, c->amgZero, mask, b, s));  // -A a
        EF_CHECK(ef_launch_bj_apply(bs, nN, binv, mask, 1.f, b, a, 0, s));                            // D^-1
    }
    return EF_OK;
}

// per-level smoothing damping from the power-iteration norms (one transfer); the captured cycle
// graphs are dropped when a damping changes
static ef_status amg_damping_finish(ef_ctx* c, cudaStream_t s) {
    const int nL = (int)c->amg.size();
    std::vector<float> om(nL), lamq(nL);
    std::vector<double> hn(3 * (size_t)kPowerSteps * nL);
    EF_CUDA(cudaMemcpyAsync(hn.data(), c->amgNorms, sizeof(double) * hn.size(), cudaMemcpyDeviceToHost, s));
    EF_CUDA(cudaStreamSynchronize(s));
    for (int l = 0; l < nL; ++l) {
        // lambda: |D^-1 A a| for the unit vector a of the last step
        const double n2 = hn[3 * (l * kPowerSteps + kPowerSteps - 1)];
        const double lam = n2 > 0.0 ? sqrt(n2) : 0.0;
        float w = c->amgOmega;
        if (lam > 0.0 && lam == lam && c->amgOmega * lam > 1.85)  // close to the stability limit 2
            w = std::max(1.f, std::round((float)(4.0 / (3.0 * lam)) * 64.f)) / 64.f;
        om[l] = w;
        // lambda on a grid of 2^(1/16) steps for the Chebyshev bounds (stable captured cycles)
        lamq[l] = lam > 0.0 && lam == lam ? (float)exp2(std::ceil(16.0 * log2(lam)) / 16.0) : 2.f;
    }
    if (om != c->levelOmega || (c->amgCheb && lamq != c->levelLam)) {
        c->levelOmega = om;
        c->levelLam = lamq;
        if (c->vcGraph) {
            cudaGraphExecDestroy(c->vcGraph);
            c->vcGraph = nullptr;
        }
        if (c->nnGraph) {
            cudaGraphExecDestroy(c->nnGraph);
            c->nnGraph = nullptr;
        }
    }
    return EF_OK;
}

static ef_status amg_damping(ef_ctx* c, cudaStream_t s) {
    EF_CHECK(amg_power_alloc(c));
    for (int l = 0; l < (int)c->amg.size(); ++l) EF_CHECK(amg_power(c, l, s));
    return amg_damping_finish(c, s);
}

// edge weights of the learned correction for the current system; only while something reads them
// (the correction is applied, or training pairs are collected): otherwise they stay stale and the
// next reader refreshes them first
ef_status nn_edge_refresh(ef_ctx* c, cudaStream_t s, bool force) {
    if (!c->nnInit || !c->nnEdgeStale) return EF_OK;
    if (!force && !c->nnOn && !(c->nnEvery > 0 && c->nnMaxPerSolve > 0)) return EF_OK;
    EF_CHECK(ef_launch_edge_weights((int)c->nNodes, c->dRowPtr, c->dColIdx, (const float*)c->dBsrVals, c->nnA, s));
    EF_CHECK(ef_launch_gather_f32(c->nBlocks, c->nnTpos, c->nnA, c->nnAT, s));
    c->nnEdgeStale = false;
    return EF_OK;
}

// dead coarse DOFs from the current Dirichlet mask, then Galerkin values, block inverses, the
// coarsest inverse and the smoothing damping for the current fine system
ef_status amg_refresh(ef_ctx* c, cudaStream_t s) {
    EF_CHECK(sell_refresh(c, s));
    if (!c->amgStale) return EF_OK;
    if (!c->amgMaskChanged && c->amgReuseLeft > 0) {
        // lagged coarse levels: the prolongators, coarse operators and damping of an earlier system
        // of the same pattern and mask; the fine level (blocks, block inverses, BF16 copy) is the
        // current system's
        c->amgReuseLeft--;
        if (c->dBsrValsH)
            EF_CHECK(ef_launch_to_bf16_split(c->nBlocks, (const float*)c->dBsrVals, c->dBsrValsH, s));
        c->amgStale = false;
        return nn_edge_refresh(c, s);
    }
    c->amgReuseLeft = c->amgMaxReuse;
    const int BCo = ef_amg_coarse_dofs();
    if (c->amgMaskChanged || !c->amgDeadValid) {
        // the dead coarse DOFs depend on the Dirichlet mask and the (fixed) aggregation only
        const uint8_t* fineDead = c->hMask.data();
        for (size_t l = 0; l < c->amg.size(); ++l) {
            AmgLevel& L = c->amg[l];
            amg_dead_mask(L, l == 0 ? 3 : BCo, fineDead, L.hDead);
            EF_CUDA(cudaMemcpyAsync(L.dead, L.hDead.data(), L.hDead.size(), cudaMemcpyHostToDevice, s));
            fineDead = L.hDead.data();
        }
        c->amgDeadValid = true;
    }
    c->amgMaskChanged = false;
    if (c->amgSmoothed) EF_CHECK(amg_power_alloc(c));
    // with reuse enabled, the damping estimates (lambda_max of D^-1 A per level) come from the
    // increment's first build; the later builds of the increment keep them
    const bool power = c->amgPowerDue || c->amgMaxReuse == 0;
    c->amgPowerDue = false;
    for (size_t l = 0; l < c->amg.size(); ++l) {
        AmgLevel& L = c->amg[l];
        const bool fine = l == 0;
        const int32_t* fRob = fine ? c->dRowOfBlock0 : c->amg[l - 1].rowOfBlock;
        const int32_t* fCol = fine ? c->dColIdx : c->amg[l - 1].colIdx;
        const float* fVals = fine ? (const float*)c->dBsrVals : c->amg[l - 1].vals;
        const uint8_t* fMask = fine ? c->dMask : c->amg[l - 1].dead;
        if (c->amgSmoothed) {
            // smoothed prolongator P = P_t - 4 / (3 lambda) D^-1 A P_t of the finer level (its lambda
            // from the power iteration on the device), then A P and P^T A P
            const float* fBinv = fine ? (const float*)c->dBinv : c->amg[l - 1].binv;
            const int nFiner = fine ? (int)c->nNodes : c->amg[l - 1].nN;
            if (power) EF_CHECK(amg_power(c, (int)l, s));
            EF_CHECK(ef_launch_sa_damping(c->amgNorms + 3 * ((int)l * kPowerSteps + kPowerSteps - 1), L.saW, s));
            EF_CHECK(ef_launch_sa_setup(fine ? 3 : BCo, L.saNP, L.saPRow, L.saPCol, L.saPSeg, L.saPSrc, L.saNAP,
                                        L.saApRow, L.saApSeg, L.saApK, L.saApP, fCol, fVals, fMask, L.offs, L.agg,
                                        fBinv, L.saW, L.saPv, L.saAPv, L.nBlocks, L.saCSeg, L.saCP, L.saCAP,
                                        L.rowOfBlock, L.colIdx, L.dead, L.vals, nFiner, L.saApRowPtr, L.saApCap, s));
            if (L.saOnePass && L.saPTh0)
                EF_CHECK(ef_launch_sa_block_copy_h(L.saNP, L.saTIdx, L.saPv, L.saPTh0, L.saPTh1, L.saPTh2, s));
            else if (L.saOnePass)
                EF_CHECK(ef_launch_sa_block_copy(fine ? 3 : BCo, L.saNP, L.saTIdx, L.saPv, L.saPT, s));
        } else {
            EF_CHECK(ef_launch_galerkin(fine ? 3 : BCo, L.nBlocks, L.gseg, L.gsrc, fRob, fCol, fVals, fMask, L.offs,
                                        L.rowOfBlock, L.colIdx, L.dead, L.vals, s));
        }
        EF_CHECK(ef_launch_bj6_setup(L.nN, L.diagPos, L.vals, L.binv, s));
        if (L.valsB) EF_CHECK(ef_launch_scale_blocks6(L.nBlocks, L.colIdx, L.vals, L.binv, L.dead, L.valsB, s));
        if (L.valsH) EF_CHECK(ef_launch_to_bf16(L.nBlocks * BCo * BCo, L.vals, L.valsH, s));
    }
    const AmgLevel& C = c->amg.back();
    EF_CHECK(ef_launch_coarsest_inverse(C.nN, C.rowPtr, C.colIdx, C.vals, c->amgCoarsestInv, s));
    if (c->dBsrValsH)
        EF_CHECK(ef_launch_to_bf16_split(c->nBlocks, (const float*)c->dBsrVals, c->dBsrValsH, s));
    if (power) {
        if (c->amgSmoothed) {
            EF_CHECK(amg_damping_finish(c, s));  // every level's power iteration ran above
        } else {
            EF_CHECK(amg_damping(c, s));
        }
    }
    if (c->postSlots > 0) {
        // C = a (I - w D^-1 A) P of the fine level for the fused post-smoothing (with the damping
        // of this build; lagged, like P, when later systems reuse the coarse levels)
        const AmgLevel& F0 = c->amg[0];
        const float w0 = c->levelOmega.empty() ? c->amgOmega : c->levelOmega[0];
        EF_CHECK(ef_launch_sa_post_setup(c->postSlots, c->dPostSrc, F0.saApRow, c->dPostApToP, F0.saPv, F0.saAPv,
                                         (const float*)c->dBinv, w0, c->amgAlpha, c->dPostQ0, c->dPostQ1,
                                         c->dPostQ2, s));
    }
    for (size_t l = 1; l < c->amg.size(); ++l) {  // the same for the 6-DOF levels
        const AmgLevel& L = c->amg[l];
        if (!L.postC) continue;
        const float wl = l < c->levelOmega.size() ? c->levelOmega[l] : c->amgOmega;
        EF_CHECK(ef_launch_sa_post6_setup(L.saNAP, L.saApRow, L.postApToP, L.saPv, L.saAPv, c->amg[l - 1].binv, wl,
                                          c->amgAlpha, L.postC, s));
    }
    c->amgStale = false;
    return nn_edge_refresh(c, s);
}

// x = V-cycle(r) on level l (l = 0: the fine system); one damped block-Jacobi sweep before and
// after the coarse correction, dense solve on the coarsest level
ef_status amg_vcycle(ef_ctx* c, int l, const float* r, float* x, cudaStream_t s) {
    const float omega = l < (int)c->levelOmega.size() ? c->levelOmega[l] : c->amgOmega;
    const int nL = (int)c->amg.size();
    const int BCo = ef_amg_coarse_dofs();
    if (l == nL) {
        const AmgLevel& C = c->amg.back();
        return ef_launch_coarsest_apply(BCo * C.nN, c->amgCoarsestInv, r, C.dead, x, s);
    }
    const bool fine = l == 0;
    const int bs = fine ? 3 : BCo;
    const int nN = fine ? (int)c->nNodes : c->amg[l - 1].nN;
    const int32_t* rowPtr = fine ? c->dRowPtr : c->amg[l - 1].rowPtr;
    const int32_t* colIdx = fine ? c->dColIdx : c->amg[l - 1].colIdx;
    const float* vals = fine ? (const float*)c->dBsrVals : c->amg[l - 1].vals;
    const float* binv = fine ? (const float*)c->dBinv : c->amg[l - 1].binv;
    const uint8_t* mask = fine ? c->dMask : c->amg[l - 1].dead;
    float* t = fine ? c->fineT : c->amg[l - 1].t;
    const void* valsH = fine ? nullptr : c->amg[l - 1].valsH;
    AmgLevel& Cn = c->amg[l];
    // fine level from a BF16 copy: the sliced-ELL one, else the BSR split copy (staged through
    // shared memory when the chunks fit)
    const bool fineH = fine && c->amgBf16 && (c->sellMode == 1 || c->dBsrValsH);
    auto fine_bf16 = [&](const float* xin, float* out, const float* bj, float om) -> ef_status {
        if (c->sellMode == 1)
            return ef_launch_sell_level3_bf16(nN, c->sellSlices, c->dSellOff, c->dSellPerm, c->dSellCol, c->dSellV8,
                                              c->dSellV1, xin, r, mask, out, bj, om, c->sellSplit, s, 1.f,
                                              c->dSellDia);
        if (c->stageCap > 0)
            return ef_launch_level_residual_bf16_staged(c->nSM, c->stageCap, nN, c->nBlocks, rowPtr, colIdx,
                                                        c->dBsrValsH, xin, r, mask, out, s, bj, om);
        return ef_launch_level_residual_bf16(nN, c->nBlocks, rowPtr, colIdx, c->dBsrValsH, xin, r, mask, out, s, bj,
                                             om);
    };
    auto residual = [&]() -> ef_status {
        if (fineH) return fine_bf16(x, t, nullptr, 0.f);
        return ef_launch_level_residual(bs, nN, rowPtr, colIdx, vals, x, r, mask, t, s, nullptr, 0.f, valsH);
    };
    // Chebyshev smoothing of degree amgSweeps on [lmax / 30, 1.1 lmax] of D^-1 A; from zero the
    // first residual is r itself
    auto chebyshev = [&](bool fromZero) -> ef_status {
        const double up = 1.1 * (l < (int)c->levelLam.size() ? c->levelLam[l] : 2.0), lo = up / 30.0;
        const double theta = 0.5 * (up + lo), delta = 0.5 * (up - lo), sigma = theta / delta;
        double rhoOld = 1.0 / sigma;
        float* d = c->chebD[l];
        if (fromZero) {
            EF_CHECK(ef_launch_cheb_step(bs, nN, binv, mask, 0.f, (float)(1.0 / theta), r, d, x, 1, s));
        } else {
            EF_CHECK(residual());
            EF_CHECK(ef_launch_cheb_step(bs, nN, binv, mask, 0.f, (float)(1.0 / theta), t, d, x, 0, s));
        }
        for (int k = 1; k < c->amgSweeps; ++k) {
            const double rho = 1.0 / (2.0 * sigma - rhoOld);
            EF_CHECK(residual());
            EF_CHECK(ef_launch_cheb_step(bs, nN, binv, mask, (float)(rho * rhoOld), (float)(2.0 * rho / delta), t, d,
                                         x, 0, s));
            rhoOld = rho;
        }
        return EF_OK;
    };
    // one fused damped block-Jacobi sweep xout = xin + omega D^-1 (r - A xin)
    auto sweep = [&](const float* xin, float* xout) -> ef_status {
        if (fineH) return fine_bf16(xin, xout, binv, omega);
        return ef_launch_level_residual(bs, nN, rowPtr, colIdx, vals, xin, r, mask, xout, s, binv, omega, valsH);
    };
    // The sweeps (the first from zero) alternate between x and a second vector; the first goes
    // to the second vector when their total count is even, so that the last one lands in x.
    // Without pre-smoothing the iterate starts as zeros in the vector the first sweep would write.
    float* x2 = fine ? c->fineX : c->amg[l - 1].x2;
    const int nPre = fine ? c->amgPre : c->amgPreC, nPost = fine ? c->amgPost : c->amgPostC;
    float* cur = x;
    if (!c->amgCheb) cur = ((std::max(nPre, 1) + nPost) & 1) ? x : x2;
    // Fused cycle (one sweep before and after, from zero): x1 = w M D^-1 r, t = r - A x1, the
    // coarse correction e of the restricted t, then x = w D^-1 (r + t) + C e in one pass (the
    // prolongation and the post-sweep).  With B = A (M D^-1) kept beside A (a scaled BF16 copy on
    // the fine level, FP32 on a 6-DOF level) t = r - w B r needs no pre-sweep launch.
    const int repsC = (l > 0 && l <= c->amgWLevels && c->amgCycle > 1) ? c->amgCycle : 1;
    const bool fusedFine = fine && c->postSlots > 0 && fineH && c->sellMode == 1 && !c->amgCheb && nPre == 1 &&
                           nPost == 1 && c->amgSmoothed;
    const bool fusedCoarse = !fine && Cn.postC && !c->amgCheb && nPre == 1 && nPost == 1 && repsC == 1 &&
                             c->amgSmoothed && l != c->clusterLevel;
    if (fusedFine || fusedCoarse) {
        const float* valsB = fine ? nullptr : c->amg[l - 1].valsB;
        if (fusedFine && c->sellScaled) {
            EF_CHECK(ef_launch_sell_level3_bf16(nN, c->sellSlices, c->dSellOff, c->dSellPerm, c->dSellCol,
                                                c->dSellV8, c->dSellV1, r, r, mask, t, nullptr, 0.f, c->sellSplit, s,
                                                omega, c->dSellDia));
        } else if (fusedCoarse && valsB) {
            EF_CHECK(ef_launch_level_residual(bs, nN, rowPtr, colIdx, valsB, r, r, mask, t, s, nullptr, 0.f, nullptr,
                                              omega));
        } else {
            EF_CHECK(ef_launch_bj_apply(bs, nN, binv, mask, omega, r, x2, 0, s));
            EF_CHECK(fusedFine ? fine_bf16(x2, t, nullptr, 0.f)
                               : ef_launch_level_residual(bs, nN, rowPtr, colIdx, vals, x2, r, mask, t, s, nullptr,
                                                          0.f, valsH));
        }
        if (Cn.saOnePass && Cn.saPTh0)
            EF_CHECK(ef_launch_sa_restrict_onepass_h(Cn.nN, Cn.saTPtr, Cn.saRowT, Cn.saPTh0, Cn.saPTh1, Cn.saPTh2, t,
                                                     Cn.dead, Cn.r, s));
        else if (Cn.saOnePass)
            EF_CHECK(ef_launch_sa_restrict_onepass(bs, Cn.nN, Cn.saTPtr, Cn.saRowT, Cn.saPT, t, Cn.dead, Cn.r, s));
        else
            EF_CHECK(ef_launch_sa_restrict2(bs, Cn.nN, Cn.saNP, Cn.saTPtr, Cn.saTIdx, Cn.saPRow, Cn.saPv, t,
                                            Cn.dead, Cn.saC, Cn.r, s));
        EF_CHECK(amg_vcycle(c, l + 1, Cn.r, Cn.x, s));
        if (fusedFine)
            return ef_launch_sa_post_fused(nN, c->postSlices, c->dPostOff, c->dPostPerm, c->dPostCol, c->dPostQ0,
                                           c->dPostQ1, c->dPostQ2, Cn.x, r, t, binv, mask, omega, x, c->sellSplit, s);
        return ef_launch_sa_post6_fused(nN, Cn.postRowPtr, Cn.postCol, Cn.postC, Cn.x, r, t, binv, mask, omega, x,
                                        s);
    }
    // pre-smoothing from zero
    if (c->amgCheb) {
        EF_CHECK(chebyshev(true));
    } else if (nPre == 0) {
        EF_CUDA(cudaMemsetAsync(cur, 0, sizeof(float) * (size_t)bs * nN, s));
    } else {
        EF_CHECK(ef_launch_bj_apply(bs, nN, binv, mask, omega, r, cur, 0, s));
        for (int k = 1; k < nPre; ++k) {
            float* nxt = cur == x ? x2 : x;
            EF_CHECK(sweep(cur, nxt));
            cur = nxt;
        }
    }
    // coarse correction (repeated for a W-cycle below the finest level)
    const int reps = repsC;
    for (int rep = 0; rep < reps; ++rep) {
        const float* res = t;  // the residual the restriction reads: r itself while the iterate is zero
        if (!c->amgCheb && nPre == 0 && rep == 0) {
            res = r;
        } else if (!c->amgCheb) {
            EF_CHECK(fineH ? fine_bf16(cur, t, nullptr, 0.f)
                                          : ef_launch_level_residual(bs, nN, rowPtr, colIdx, vals, cur, r, mask, t, s,
                                                                     nullptr, 0.f, valsH));
        } else {
            EF_CHECK(residual());
        }
        if (l == c->clusterLevel) {
            // restriction, the whole cycle below and the prolongation as one cluster launch
            if (cur != c->clusterCur || x != c->amg[l - 1].x) {
                ef_set_error("multigrid: cluster program built for other buffers");
                return EF_ERR_ARG;
            }
            EF_CHECK(ef_launch_coarse_cycle(c->dCoarseOps, c->nCoarseOps, s));
            continue;
        }
        if (c->amgSmoothed && Cn.saOnePass && Cn.saPTh0)
            EF_CHECK(ef_launch_sa_restrict_onepass_h(Cn.nN, Cn.saTPtr, Cn.saRowT, Cn.saPTh0, Cn.saPTh1, Cn.saPTh2, res,
                                                     Cn.dead, Cn.r, s));
        else if (c->amgSmoothed && Cn.saOnePass)
            EF_CHECK(ef_launch_sa_restrict_onepass(bs, Cn.nN, Cn.saTPtr, Cn.saRowT, Cn.saPT, res, Cn.dead, Cn.r, s));
        else if (c->amgSmoothed && c->saTransfer >= 1)
            EF_CHECK(ef_launch_sa_restrict2(bs, Cn.nN, Cn.saNP, Cn.saTPtr, Cn.saTIdx, Cn.saPRow, Cn.saPv, res,
                                            Cn.dead, Cn.saC, Cn.r, s));
        else if (c->amgSmoothed)
            EF_CHECK(ef_launch_sa_restrict(bs, Cn.nN, Cn.saTPtr, Cn.saTIdx, Cn.saPRow, Cn.saPv, res, Cn.dead, Cn.r,
                                           s));
        else
            EF_CHECK(ef_launch_restrict(bs, Cn.nN, Cn.aggPtr, Cn.aggIdx, Cn.offs, res, Cn.dead, Cn.r, s));
        EF_CHECK(amg_vcycle(c, l + 1, Cn.r, Cn.x, s));
        if (c->amgSmoothed && Cn.saOnePass)
            EF_CHECK(ef_launch_sa_prolong_onepass(bs, nN, Cn.saCap, Cn.saPRowPtr, Cn.saPCol, Cn.saPv, Cn.x, mask, cur,
                                                  c->amgAlpha, s));
        else if (c->amgSmoothed && c->saTransfer >= 1)
            EF_CHECK(ef_launch_sa_prolong2(bs, nN, Cn.saNP, Cn.saPRowPtr, Cn.saPCol, Cn.saPv, Cn.x, mask, Cn.saC, cur,
                                           c->amgAlpha, s));
        else if (c->amgSmoothed)
            EF_CHECK(ef_launch_sa_prolong(bs, nN, Cn.saPRowPtr, Cn.saPCol, Cn.saPv, Cn.x, mask, cur, c->amgAlpha, s));
        else
            EF_CHECK(ef_launch_prolong(bs, nN, Cn.agg, Cn.offs, Cn.x, mask, cur, s, c->amgAlpha));
    }
    // post-smoothing
    if (c->amgCheb) {
        EF_CHECK(chebyshev(false));
    } else {
        for (int k = 0; k < nPost; ++k) {
            float* nxt = cur == x ? x2 : x;
            EF_CHECK(sweep(cur, nxt));
            cur = nxt;
        }
        if (cur != x) {
            ef_set_error("multigrid: smoothing sweeps did not end in the output vector");
            return EF_ERR_ARG;
        }
    }
    return EF_OK;
}

// preconditioner of FGMRES: z = V-cycle(v) (+ the learned correction when enabled)
// learned correction with Mv in vcOut and v in vcIn: rho = v - K Mv, N = NN([Mv, rho, D^-1 rho]),
// z = Mv + alpha N with the alpha that minimises |v - K z| (never worse than Mv alone in that
// norm); z in vcOut2
