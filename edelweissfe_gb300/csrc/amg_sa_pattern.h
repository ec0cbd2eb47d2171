// Index maps of smoothed aggregation (host code, plain C++).
//
// For one level transition of the multigrid: a finer block pattern (rowPtr, colIdx; nF block rows
// of BF DOFs) and its aggregation agg[nF] -> [0, nC).  The tentative prolongator P_t has one
// BF x 6 block per finer node m, in column agg(m) (rigid-body modes of the aggregate); the
// smoothed prolongator is
//     P = P_t - w D^-1 A P_t,   block (m, J) = [J == agg(m)] P_t(m) - w D_m^-1 sum_{k in row m,
//                                                 agg(col(k)) == J} A_k P_t(col(k)),
// the product AP = A P has blocks (m, J) = sum_{k in row m} A_k P(col(k), J), and the Galerkin
// operator A_c = P^T A P has blocks (I, J) = sum_m P(m, I)^T AP(m, J).  These maps list, in a
// fixed order, which blocks enter each of those sums, so that the device kernels compute them
// as deterministic segmented sums without atomics.  All lists are sorted: rows by increasing
// column, contributions by increasing source index.
#pragma once

#include <stdint.h>

#include <algorithm>
#include <vector>

namespace ef {

struct SAPattern {
    int nF = 0, nC = 0;
    // P: block rows of the finer level, columns = coarse nodes
    std::vector<int32_t> pRowPtr, pCol;   // [nF + 1], [nnzP]
    std::vector<int32_t> pRow;            // [nnzP] block row of each P block
    std::vector<int64_t> pSeg;            // [nnzP + 1] into pSrc
    std::vector<int32_t> pSrc;            // finer blocks k of row m with agg(col(k)) == J
    // P^T by coarse node: the P blocks of column I in increasing block row
    std::vector<int32_t> tPtr, tIdx;      // [nC + 1], [nnzP]
    // AP: block rows of the finer level, columns = coarse nodes
    std::vector<int32_t> apRowPtr, apCol; // [nF + 1], [nnzAP]
    std::vector<int64_t> apSeg;           // [nnzAP + 1] into apK / apP
    std::vector<int32_t> apK, apP;        // pairs (finer block k, P block (col(k), J))
    // coarse pattern and the Galerkin map
    std::vector<int32_t> cRowPtr, cCol;   // [nC + 1], [nnzC]
    std::vector<int64_t> cSeg;            // [nnzC + 1] into cP / cAP
    std::vector<int32_t> cP, cAP;         // pairs (P block (m, I), AP block (m, J)), m increasing
};

// binary search of column c in the sorted row [b, e) of cols; -1 when absent
inline int64_t sa_find(const std::vector<int32_t>& cols, int64_t b, int64_t e, int32_t c) {
    const int32_t* p = std::lower_bound(cols.data() + b, cols.data() + e, c);
    return (p != cols.data() + e && *p == c) ? (int64_t)(p - cols.data()) : -1;
}

inline void build_sa_pattern(int nF, const int32_t* rowPtr, const int32_t* colIdx, const int32_t* agg, int nC,
                             SAPattern& S) {
    S.nF = nF;
    S.nC = nC;
    // ---- P pattern: row m has the aggregates of its neighbours (itself included) ----
    S.pRowPtr.assign(nF + 1, 0);
    S.pCol.clear();
    std::vector<int32_t> tmp;
    for (int m = 0; m < nF; ++m) {
        tmp.clear();
        tmp.push_back(agg[m]);
        for (int32_t k = rowPtr[m]; k < rowPtr[m + 1]; ++k) tmp.push_back(agg[colIdx[k]]);
        std::sort(tmp.begin(), tmp.end());
        tmp.erase(std::unique(tmp.begin(), tmp.end()), tmp.end());
        S.pCol.insert(S.pCol.end(), tmp.begin(), tmp.end());
        S.pRowPtr[m + 1] = (int32_t)S.pCol.size();
    }
    const int64_t nnzP = (int64_t)S.pCol.size();
    S.pRow.resize(nnzP);
    for (int m = 0; m < nF; ++m)
        for (int32_t b = S.pRowPtr[m]; b < S.pRowPtr[m + 1]; ++b) S.pRow[b] = m;
    // contributions of block (m, J): the finer blocks k of row m with agg(col k) == J, in k order
    S.pSeg.assign(nnzP + 1, 0);
    for (int m = 0; m < nF; ++m)
        for (int32_t k = rowPtr[m]; k < rowPtr[m + 1]; ++k) {
            const int64_t b = sa_find(S.pCol, S.pRowPtr[m], S.pRowPtr[m + 1], agg[colIdx[k]]);
            S.pSeg[b + 1]++;
        }
    for (int64_t b = 0; b < nnzP; ++b) S.pSeg[b + 1] += S.pSeg[b];
    S.pSrc.assign(S.pSeg[nnzP], 0);
    {
        std::vector<int64_t> fill(S.pSeg.begin(), S.pSeg.end() - 1);
        for (int m = 0; m < nF; ++m)
            for (int32_t k = rowPtr[m]; k < rowPtr[m + 1]; ++k) {
                const int64_t b = sa_find(S.pCol, S.pRowPtr[m], S.pRowPtr[m + 1], agg[colIdx[k]]);
                S.pSrc[fill[b]++] = k;
            }
    }
    // ---- P^T: blocks of each coarse column in increasing row ----
    S.tPtr.assign(nC + 1, 0);
    for (int64_t b = 0; b < nnzP; ++b) S.tPtr[S.pCol[b] + 1]++;
    for (int I = 0; I < nC; ++I) S.tPtr[I + 1] += S.tPtr[I];
    S.tIdx.assign(nnzP, 0);
    {
        std::vector<int32_t> fill(S.tPtr.begin(), S.tPtr.end() - 1);
        for (int64_t b = 0; b < nnzP; ++b) S.tIdx[fill[S.pCol[b]]++] = (int32_t)b;  // rows increase with b
    }
    // ---- AP pattern: row m has the P columns of its neighbours' P rows ----
    S.apRowPtr.assign(nF + 1, 0);
    S.apCol.clear();
    for (int m = 0; m < nF; ++m) {
        tmp.clear();
        for (int32_t k = rowPtr[m]; k < rowPtr[m + 1]; ++k) {
            const int n = colIdx[k];
            for (int32_t b = S.pRowPtr[n]; b < S.pRowPtr[n + 1]; ++b) tmp.push_back(S.pCol[b]);
        }
        std::sort(tmp.begin(), tmp.end());
        tmp.erase(std::unique(tmp.begin(), tmp.end()), tmp.end());
        S.apCol.insert(S.apCol.end(), tmp.begin(), tmp.end());
        S.apRowPtr[m + 1] = (int32_t)S.apCol.size();
    }
    const int64_t nnzAP = (int64_t)S.apCol.size();
    S.apSeg.assign(nnzAP + 1, 0);
    for (int m = 0; m < nF; ++m)
        for (int32_t k = rowPtr[m]; k < rowPtr[m + 1]; ++k) {
            const int n = colIdx[k];
            for (int32_t b = S.pRowPtr[n]; b < S.pRowPtr[n + 1]; ++b) {
                const int64_t a = sa_find(S.apCol, S.apRowPtr[m], S.apRowPtr[m + 1], S.pCol[b]);
                S.apSeg[a + 1]++;
            }
        }
    for (int64_t a = 0; a < nnzAP; ++a) S.apSeg[a + 1] += S.apSeg[a];
    S.apK.assign(S.apSeg[nnzAP], 0);
    S.apP.assign(S.apSeg[nnzAP], 0);
    {
        std::vector<int64_t> fill(S.apSeg.begin(), S.apSeg.end() - 1);
        for (int m = 0; m < nF; ++m)
            for (int32_t k = rowPtr[m]; k < rowPtr[m + 1]; ++k) {
                const int n = colIdx[k];
                for (int32_t b = S.pRowPtr[n]; b < S.pRowPtr[n + 1]; ++b) {
                    const int64_t a = sa_find(S.apCol, S.apRowPtr[m], S.apRowPtr[m + 1], S.pCol[b]);
                    S.apK[fill[a]] = k;
                    S.apP[fill[a]] = b;
                    fill[a]++;
                }
            }
    }
    // ---- coarse pattern: (I, J) for every m with P(m, I) and AP(m, J) ----
    std::vector<std::vector<int32_t>> cols(nC);
    for (int I = 0; I < nC; ++I) {
        auto& v = cols[I];
        for (int32_t t = S.tPtr[I]; t < S.tPtr[I + 1]; ++t) {
            const int m = S.pRow[S.tIdx[t]];
            for (int32_t a = S.apRowPtr[m]; a < S.apRowPtr[m + 1]; ++a) v.push_back(S.apCol[a]);
        }
        std::sort(v.begin(), v.end());
        v.erase(std::unique(v.begin(), v.end()), v.end());
    }
    S.cRowPtr.assign(nC + 1, 0);
    S.cCol.clear();
    for (int I = 0; I < nC; ++I) {
        S.cCol.insert(S.cCol.end(), cols[I].begin(), cols[I].end());
        S.cRowPtr[I + 1] = (int32_t)S.cCol.size();
    }
    const int64_t nnzC = (int64_t)S.cCol.size();
    S.cSeg.assign(nnzC + 1, 0);
    for (int I = 0; I < nC; ++I)
        for (int32_t t = S.tPtr[I]; t < S.tPtr[I + 1]; ++t) {
            const int m = S.pRow[S.tIdx[t]];
            for (int32_t a = S.apRowPtr[m]; a < S.apRowPtr[m + 1]; ++a) {
                const int64_t c = sa_find(S.cCol, S.cRowPtr[I], S.cRowPtr[I + 1], S.apCol[a]);
                S.cSeg[c + 1]++;
            }
        }
    for (int64_t c = 0; c < nnzC; ++c) S.cSeg[c + 1] += S.cSeg[c];
    S.cP.assign(S.cSeg[nnzC], 0);
    S.cAP.assign(S.cSeg[nnzC], 0);
    {
        std::vector<int64_t> fill(S.cSeg.begin(), S.cSeg.end() - 1);
        for (int I = 0; I < nC; ++I)
            for (int32_t t = S.tPtr[I]; t < S.tPtr[I + 1]; ++t) {  // m increasing
                const int32_t pb = S.tIdx[t];
                const int m = S.pRow[pb];
                for (int32_t a = S.apRowPtr[m]; a < S.apRowPtr[m + 1]; ++a) {
                    const int64_t c = sa_find(S.cCol, S.cRowPtr[I], S.cRowPtr[I + 1], S.apCol[a]);
                    S.cP[fill[c]] = pb;
                    S.cAP[fill[c]] = a;
                    fill[c]++;
                }
            }
    }
}

}  // namespace ef
