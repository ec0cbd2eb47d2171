// C ABI of the efgpu library: context and model setup (element groups, DOF maps, VIJ -> CSR slot
// maps and the 3x3-block pattern built on the host), the element loop and its state, element
// results.  The system, solver, multigrid, learned-correction and batch entry points are in
// system.cu, solve.cu, precond.cu, learned_api.cu and batch_api.cu.

#include "ctx.h"

// launch counter (see ef_common.cuh); launches issued during a stream capture are credited to the
// graph being captured on this thread instead
static std::atomic<long long> g_launchCount{0};
thread_local long long* t_captureCount = nullptr;
void ef::note_launches(long long n) {
    if (t_captureCount)
        *t_captureCount += n;
    else
        g_launchCount.fetch_add(n, std::memory_order_relaxed);
}
long long ef::launches() { return g_launchCount.load(std::memory_order_relaxed); }

// programmatic dependent launch of the iteration kernels (EF_PDL=0 turns it off): on the
// 160k-element J2 box 0.1239 against 0.1265 s per load step
bool ef::dep_launch_enabled() {
    static const bool on = [] {
        const char* e = getenv("EF_PDL");
        return !e || atoi(e) != 0;
    }();
    return on;
}


static thread_local std::string g_err;
void ef_set_error(const std::string& s) { g_err = s; }

namespace {

struct TypeInfo {
    const char* name;
    int nNodes;
    int rule;  // 0: 1 point, 1: 2x2x2, 2: 3x3x3
    int tl;
};

// elements/library.py:212-291 (small strain), :453-532 (total Lagrange) and the aliases of :535-551
const TypeInfo kTypes[] = {
    {"C3D8", 8, 1, 0},    {"C3D8R", 8, 0, 0},   {"C3D8E", 8, 2, 0},    {"C3D20", 20, 2, 0},
    {"C3D20R", 20, 1, 0}, {"C3D8TL", 8, 1, 1},  {"C3D20TL", 20, 2, 1}, {"C3D8RTL", 8, 0, 1},
    {"C3D8ETL", 8, 2, 1}, {"C3D20RTL", 20, 1, 1}, {"C3D8N", 8, 1, 0},  {"C3D20N", 20, 2, 0},
    {"C3D8NTL", 8, 1, 1}, {"C3D20NTL", 20, 2, 1},
};

bool ieq(const char* a, const char* b) {
    for (; *a && *b; ++a, ++b)
        if (tolower(*a) != tolower(*b)) return false;
    return *a == *b;
}

// parametric node tables (S1, S2, S3) -- elements/displacementelement/_elementcomputationmatrices.py _J3D8/_J3D20
const int kHex8[8][3] = {{-1, -1, -1}, {-1, -1, 1}, {1, -1, 1}, {1, -1, -1},
                         {-1, 1, -1},  {-1, 1, 1},  {1, 1, 1},  {1, 1, -1}};
const int kHex20[20][3] = {{-1, -1, -1}, {-1, -1, 1}, {1, -1, 1}, {1, -1, -1}, {-1, 1, -1}, {-1, 1, 1}, {1, 1, 1},
                           {1, 1, -1},   {-1, -1, 0}, {0, -1, 1}, {1, -1, 0},  {0, -1, -1}, {-1, 1, 0}, {0, 1, 1},
                           {1, 1, 0},    {0, 1, -1},  {-1, 0, -1}, {-1, 0, 1}, {1, 0, 1},   {1, 0, -1}};

// Gauss rules of elements/library.py (xi, eta, zeta, w)
void gauss_rule(int rule, std::vector<double>& xi, std::vector<double>& eta, std::vector<double>& zeta,
                std::vector<double>& w) {
    xi.clear();
    eta.clear();
    zeta.clear();
    w.clear();
    if (rule == 0) {
        xi = {0.0};
        eta = {0.0};
        zeta = {0.0};
        w = {8.0};
    } else if (rule == 1) {
        const double g = 1.0 / sqrt(3.0);
        const double s8[4] = {-1, 1, 1, -1}, t8[4] = {-1, -1, 1, 1};
        for (int h = 0; h < 2; ++h)
            for (int i = 0; i < 4; ++i) {
                xi.push_back(h ? g : -g);
                eta.push_back(g * t8[i]);
                zeta.push_back(g * s8[i]);
                w.push_back(1.0);
            }
    } else {
        const double r = sqrt(0.6);
        const double t20[9] = {-1, -1, -1, 0, 0, 0, 1, 1, 1};
        const double s20[3] = {-1, 0, 1};
        const double w1 = pow(5.0 / 9.0, 3), w2 = pow(5.0 / 9.0, 2) * (8.0 / 9.0), w3 = (5.0 / 9.0) * pow(8.0 / 9.0, 2),
                     w4 = pow(8.0 / 9.0, 3);
        const double wI[3] = {w1, w2, w1}, wII[3] = {w2, w3, w2}, wIII[3] = {w3, w4, w3};
        const double* wrows[9] = {wI, wII, wI, wII, wIII, wII, wI, wII, wI};
        for (int h = 0; h < 3; ++h)
            for (int i = 0; i < 9; ++i) {
                xi.push_back(r * (h - 1));
                eta.push_back(r * t20[i]);
                zeta.push_back(r * s20[i % 3]);
                w.push_back(wrows[(9 * h + i) / 3][i % 3]);  // 9 groups of 3 over the 27 points
            }
    }
}

void shape(int nn, const double* S, double* N, double dN[3][20]) {
    for (int a = 0; a < nn; ++a) {
        const int* sa = nn == 8 ? kHex8[a] : kHex20[a];
        double f[3], df[3];
        for (int k = 0; k < 3; ++k) {
            if (sa[k] != 0) {
                f[k] = 1.0 + sa[k] * S[k];
                df[k] = sa[k];
            } else {
                f[k] = 1.0 - S[k] * S[k];
                df[k] = -2.0 * S[k];
            }
        }
        const bool corner = sa[0] != 0 && sa[1] != 0 && sa[2] != 0;
        if (nn == 8) {
            N[a] = f[0] * f[1] * f[2] / 8.0;
            dN[0][a] = df[0] * f[1] * f[2] / 8.0;
            dN[1][a] = f[0] * df[1] * f[2] / 8.0;
            dN[2][a] = f[0] * f[1] * df[2] / 8.0;
        } else if (corner) {
            const double lin = sa[0] * S[0] + sa[1] * S[1] + sa[2] * S[2] - 2.0;
            N[a] = f[0] * f[1] * f[2] * lin / 8.0;
            dN[0][a] = (df[0] * f[1] * f[2] * lin + f[0] * f[1] * f[2] * sa[0]) / 8.0;
            dN[1][a] = (f[0] * df[1] * f[2] * lin + f[0] * f[1] * f[2] * sa[1]) / 8.0;
            dN[2][a] = (f[0] * f[1] * df[2] * lin + f[0] * f[1] * f[2] * sa[2]) / 8.0;
        } else {
            N[a] = f[0] * f[1] * f[2] / 4.0;
            dN[0][a] = df[0] * f[1] * f[2] / 4.0;
            dN[1][a] = f[0] * df[1] * f[2] / 4.0;
            dN[2][a] = f[0] * f[1] * df[2] / 4.0;
        }
    }
}

void build_tables(const TypeInfo& t, ElemTables& T) {
    memset(&T, 0, sizeof(T));
    std::vector<double> xi, eta, zeta, w;
    gauss_rule(t.rule, xi, eta, zeta, w);
    T.nNodes = t.nNodes;
    T.nQP = (int)w.size();
    T.totalLagrange = t.tl;
    T.quirk = t.nNodes == 20 ? 1 : 0;  // both element families use _J3D20 with its row-2 term
    for (int q = 0; q < T.nQP; ++q) {
        double N[20], dN[3][20];
        const double Sb[3] = {eta[q], xi[q], zeta[q]};  // B/J evaluation point
        shape(t.nNodes, Sb, N, dN);
        for (int r = 0; r < 3; ++r)
            for (int a = 0; a < t.nNodes; ++a) {
                T.dNdS_d[q][r][a] = dN[r][a];
                T.dNdS_f[q][r][a] = (float)dN[r][a];
            }
        const double Sn[3] = {xi[q], eta[q], zeta[q]};  // computeNOperator evaluation point
        double dN2[3][20];
        shape(t.nNodes, Sn, N, dN2);
        for (int a = 0; a < t.nNodes; ++a) T.N[q][a] = N[a];
        T.w[q] = w[q];
        T.quirkFac[q] = zeta[q] - xi[q];
    }
}

int material_kind(const char* m, int* nProps) {
    if (ieq(m, "linearelastic")) {
        *nProps = 2;
        return MAT_LINEAR_ELASTIC;
    }
    if (ieq(m, "vonmises")) {
        *nProps = 6;
        return MAT_VON_MISES;
    }
    if (ieq(m, "neohookewa")) {
        *nProps = 2;
        return MAT_NEOHOOKE_WA;
    }
    return -1;
}

}  // namespace


int ef_abi_version(void) { return 3; }

const char* ef_last_error(void) { return g_err.c_str(); }

ef_status ef_create(int64_t nDof, const double* nodeCoords, ef_ctx** out) {
    if (!out || nDof <= 0 || !nodeCoords) {
        ef_set_error("ef_create: invalid arguments");
        return EF_ERR_ARG;
    }
    if (nDof % 3 != 0 || nDof >= (int64_t)1 << 31) {
        ef_set_error("ef_create: nDof must be a multiple of 3 (displacement triplets) and < 2^31");
        return EF_ERR_ARG;
    }
    ef_ctx* c = new ef_ctx();
    c->nDof = nDof;
    c->nNodes = nDof / 3;
    c->hX.assign(nodeCoords, nodeCoords + nDof);
    int dev = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&c->nSM, cudaDevAttrMultiProcessorCount, dev);
    *out = c;
    return EF_OK;
}

void ef_destroy(ef_ctx* c) {
    if (!c) return;
    auto F = [](void* p) {
        if (p) cudaFree(p);
    };
    F(c->dX);
    for (auto& g : c->groups) {
        F(g.nodeDof);
        F(g.state[0]);
        F(g.state[1]);
        F((void*)g.propsTable);
        F((void*)g.elemRow);
        F(g.geo);
        F(g.geoS);
    }
    for (auto* t : c->dTables) F(t);
    for (auto& r : c->results) {
        F(r.dEl);
        F(r.dQp);
        F(r.dTable);
    }
    F(c->Pe);
    F(c->Kblk);
    F(c->dFlags);
    F(c->dDirIdx);
    F(c->dDirMask);
    F(c->dNewton);
    F(c->dSellOff);
    F(c->dSellPerm);
    F(c->dSellCol);
    F(c->dSellDia);
    F(c->amgPowFac);
    F(c->dSellSrc);
    F(c->dSellV9);
    F(c->dSellV8);
    F(c->dSellV1);
    F(c->dPostOff);
    F(c->dPostPerm);
    F(c->dPostCol);
    F(c->dPostSrc);
    F(c->dPostApToP);
    F(c->dPostQ0);
    F(c->dPostQ1);
    F(c->dPostQ2);
    F(c->dNodeDof);
    F(c->dCondPtr);
    F(c->dCondSrc);
    F(c->dCondW);
    F(c->dBsrW);
    F(c->dTieS);
    F(c->dTieA);
    F(c->dTieB);
    F(c->dTieTmp);
    F(c->dRowPtr);
    F(c->dColIdx);
    F(c->dBsrSeg);
    F(c->dBsrSrc);
    F(c->dDiagPos);
    F(c->dBsrVals);
    F(c->dBinv);
    F(c->dMask);
    F(c->dIndptr);
    F(c->dIndices);
    F(c->dCsrSeg);
    F(c->dCsrPerm);
    F(c->dKvijTmp);
    F(c->dPart);
    F(c->dRed);
    F(c->dPartA);
    F(c->dPartB);
    F(c->dBar);
    F(c->dPcgRes);
    for (auto* p : c->w32) F(p);
    for (auto* p : c->w64) F(p);
    for (auto* p : c->w64k) F(p);
    for (auto* p : c->dTang) F(p);
    F(c->dYe);
    for (auto& L : c->amg) L.free_device();
    F(c->amgCoarsestInv);
    F(c->amgPow[0]);
    F(c->amgPow[1]);
    F(c->amgZero);
    F(c->dBsrValsH);
    for (float* p : c->chebD) F(p);
    F(c->dBatchNodePtr);
    F(c->dBatchOrder);
    F(c->vcIn);
    F(c->vcOut);
    if (c->vcGraph) cudaGraphExecDestroy(c->vcGraph);
    if (c->dCoarseOps) cudaFree(c->dCoarseOps);
    if (c->amgNorms) cudaFree(c->amgNorms);
    if (c->egExec) cudaGraphExecDestroy(c->egExec);
    if (c->nnGraph) cudaGraphExecDestroy(c->nnGraph);
    for (void* p : {(void*)c->nnP, (void*)c->nnPf, (void*)c->nnM1, (void*)c->nnM2, (void*)c->nnG, c->nnPb,
                    (void*)c->nnActs, (void*)c->nnF, (void*)c->nnWork, (void*)c->nnPart, (void*)c->nnA,
                    (void*)c->nnAT, (void*)c->nnTpos, (void*)c->nnRed, (void*)c->vcOut2})
        F(p);
    for (auto& smp : c->nnSamples)
        for (void* p : {(void*)smp.f, (void*)smp.base, (void*)smp.r, (void*)smp.e}) F(p);
    F(c->nnRho);
    F(c->nnN);
    F(c->nnKN);
    for (auto& sy : c->nnSystems) {
        F(sy.K);
        F(sy.a);
    }
    F(c->nnD);
    F(c->nnKd);
    for (float* p : c->nnSnaps) F(p);
    if (c->capStream) cudaStreamDestroy(c->capStream);
    F(c->dRowOfBlock0);
    F(c->fineX);
    F(c->fineT);
    if (c->fgPin) cudaFreeHost(c->fgPin);
    for (int k = 0; k < 2; ++k) {
        if (c->fgDone[k]) cudaEventDestroy(c->fgDone[k]);
        for (int e = 0; e < 4; ++e)
            if (c->fgEv[k][e]) cudaEventDestroy(c->fgEv[k][e]);
    }
    if (c->fgNormDone) cudaEventDestroy(c->fgNormDone);
    F(c->fgV);
    F(c->fgZ);
    F(c->fgW);
    F(c->fgPart);
    F(c->fgH);
    F(c->fgPartN);
    F(c->fgPartF);
    F(c->fgSc);
    F(c->fgTicket);
    for (auto e : c->ev)
        if (e) cudaEventDestroy(e);
    for (auto e : c->evS)
        if (e) cudaEventDestroy(e);
    delete c;
}

ef_status ef_add_group(ef_ctx* c, const char* elType, const char* material, const double* props, int nProps,
                       int nEl, const int32_t* elDofs, int* groupId) {
    if (!c || !elType || !material || nEl < 0 || (nEl > 0 && !elDofs)) {
        ef_set_error("ef_add_group: invalid arguments");
        return EF_ERR_ARG;
    }
    if (c->finalized) {
        ef_set_error("ef_add_group: context already finalized");
        return EF_ERR_STATE;
    }
    if ((int)c->hg.size() >= EF_MAX_GROUPS) {
        ef_set_error("ef_add_group: too many groups");
        return EF_ERR_ARG;
    }
    const TypeInfo* ti = nullptr;
    for (const auto& t : kTypes)
        if (ieq(t.name, elType)) ti = &t;
    if (!ti) {
        ef_set_error(std::string("ef_add_group: unknown element type ") + elType);
        return EF_ERR_ARG;
    }
    int need = 0;
    const int mk = material_kind(material, &need);
    if (mk < 0) {
        ef_set_error(std::string("ef_add_group: unknown material ") + material);
        return EF_ERR_ARG;
    }
    if (nProps < need || nProps > 8 || !props) {
        ef_set_error("ef_add_group: wrong number of material properties");
        return EF_ERR_ARG;
    }
    if ((ti->tl && mk != MAT_NEOHOOKE_WA) || (!ti->tl && mk == MAT_NEOHOOKE_WA)) {
        ef_set_error("ef_add_group: total-Lagrange elements need a hyperelastic material and vice versa");
        return EF_ERR_ARG;
    }
    HostGroup g;
    g.elType = ti->name;
    g.mat = mk;
    g.props.assign(props, props + nProps);
    g.nEl = nEl;
    g.nNodes = ti->nNodes;
    g.tl = ti->tl;
    ElemTables T;
    build_tables(*ti, T);
    g.nQP = T.nQP;
    const int nd = 3 * ti->nNodes;
    g.nodeDof.resize((size_t)nEl * ti->nNodes);
    for (int64_t e = 0; e < nEl; ++e)
        for (int a = 0; a < ti->nNodes; ++a) {
            const int32_t d0 = elDofs[e * nd + 3 * a];
            if (d0 < 0 || d0 + 2 >= c->nDof || d0 % 3 != 0 || elDofs[e * nd + 3 * a + 1] != d0 + 1 ||
                elDofs[e * nd + 3 * a + 2] != d0 + 2) {
                ef_set_error("ef_add_group: element DOFs must be in-range node triplets (3n, 3n+1, 3n+2)");
                return EF_ERR_ARG;
            }
            g.nodeDof[e * ti->nNodes + a] = d0;
        }
    ef_status st = EF_OK;
    ElemTables* dT = dalloc<ElemTables>(1, &st);
    if (!dT) return st;
    EF_CUDA(cudaMemcpy(dT, &T, sizeof(T), cudaMemcpyHostToDevice));
    c->dTables.push_back(dT);
    if (groupId) *groupId = (int)c->hg.size();
    c->hg.push_back(std::move(g));
    return EF_OK;
}

ef_status ef_set_ties(ef_ctx* c, const int64_t* slave, const int64_t* masterA, const int64_t* masterB, int64_t n) {
    if (!c) return EF_ERR_ARG;
    if (c->finalized) {
        ef_set_error("ef_set_ties: context already finalized");
        return EF_ERR_STATE;
    }
    if (n < 0 || (n > 0 && (!slave || !masterA || !masterB))) return EF_ERR_ARG;
    const int64_t nN = c->nNodes;
    std::vector<uint8_t> isSlave(nN, 0);
    for (int64_t i = 0; i < n; ++i) {
        const int64_t s_ = slave[i], a = masterA[i], b = masterB[i];
        if (s_ < 0 || s_ >= nN || a < 0 || a >= nN || b < 0 || b >= nN || s_ == a || s_ == b || isSlave[s_]) {
            ef_set_error("ef_set_ties: node out of range, self-tied or tied twice");
            return EF_ERR_ARG;
        }
        isSlave[s_] = 1;
    }
    for (int64_t i = 0; i < n; ++i)
        if (isSlave[masterA[i]] || isSlave[masterB[i]]) {
            ef_set_error("ef_set_ties: a master node is itself tied");
            return EF_ERR_ARG;
        }
    c->hTieS.assign(slave, slave + n);
    c->hTieA.assign(masterA, masterA + n);
    c->hTieB.assign(masterB, masterB + n);
    return EF_OK;
}

// slots 6 and 7 of a small-strain material's property row: lambda and G of (E, nu), formed once
// (the element kernel reads them instead of dividing per Gauss point)
static void derived_props(int mat, double* p) {
    if (mat != MAT_LINEAR_ELASTIC && mat != MAT_VON_MISES) return;
    const double E = p[0], nu = p[1];
    p[6] = E * nu / ((1.0 + nu) * (1.0 - 2.0 * nu));
    p[7] = E / (2.0 * (1.0 + nu));
}

ef_status ef_set_group_cutback(ef_ctx* c, int groupId, double scale) {
    if (!c) return EF_ERR_ARG;
    if (c->finalized) {
        ef_set_error("ef_set_group_cutback: context already finalized");
        return EF_ERR_STATE;
    }
    if (groupId < 0 || groupId >= (int)c->hg.size() || !(scale > 0.0 && scale < 1.0)) {
        ef_set_error("ef_set_group_cutback: needs a group and a scale in (0, 1)");
        return EF_ERR_ARG;
    }
    c->hg[groupId].cutback = scale;
    return EF_OK;
}

ef_status ef_set_group_props(ef_ctx* c, int groupId, const double* table, int nRows, int nProps,
                             const int32_t* elemRow) {
    if (!c) return EF_ERR_ARG;
    if (c->finalized) {
        ef_set_error("ef_set_group_props: context already finalized");
        return EF_ERR_STATE;
    }
    if (groupId < 0 || groupId >= (int)c->hg.size() || !table || !elemRow || nRows <= 0 || nProps <= 0 ||
        nProps > 8) {
        ef_set_error("ef_set_group_props: bad arguments");
        return EF_ERR_ARG;
    }
    HostGroup& h = c->hg[groupId];
    int need = 0;
    const char* names[3] = {"linearelastic", "vonmises", "neohookewa"};
    material_kind(names[h.mat], &need);
    if (nProps < need) {
        ef_set_error("ef_set_group_props: too few material properties per row");
        return EF_ERR_ARG;
    }
    h.propsTable.assign((size_t)nRows * 8, 0.0);
    for (int r = 0; r < nRows; ++r) {
        for (int i = 0; i < nProps; ++i) h.propsTable[(size_t)r * 8 + i] = table[(size_t)r * nProps + i];
        derived_props(h.mat, &h.propsTable[(size_t)r * 8]);
    }
    h.elemRow.assign(elemRow, elemRow + h.nEl);
    for (int32_t r : h.elemRow)
        if (r < 0 || r >= nRows) {
            ef_set_error("ef_set_group_props: element row out of range");
            h.propsTable.clear();
            h.elemRow.clear();
            return EF_ERR_ARG;
        }
    return EF_OK;
}

ef_status ef_finalize(ef_ctx* c, int options) {
    if (!c) return EF_ERR_ARG;
    if (c->finalized) {
        ef_set_error("ef_finalize: called twice");
        return EF_ERR_STATE;
    }
    c->keFp64 = (options & EF_OPT_KE_FP64) ? 1 : 0;
    c->scalar = !(options & EF_OPT_NO_SCALAR_CSR) && c->hTieS.empty();  // the reference CSR has no ties
    if (const char* e = getenv("EF_ELEM_GRAPH")) c->elemGraphs = atoi(e) != 0;
    if (const char* e = getenv("EF_FGMRES_HOLD")) c->fgHold = std::max(0.0, atof(e));
    if (const char* e = getenv("EF_REFINE_AIM")) {
        const double v = atof(e);
        if (v > 0.0 && v <= 1.0) c->refineAim = v;
    }
    if (const char* e = getenv("EF_REFINE_FLOOR")) {
        const double v = atof(e);
        if (v >= 0.0 && v < 0.5) c->refineFloor = v;
    }
    if (const char* e = getenv("EF_MPNN_TC")) c->nnTensorCores = atoi(e) != 0;
    const size_t ks = c->keFp64 ? sizeof(double) : sizeof(float);
    ef_status st = EF_OK;
    const int64_t nNodes = c->nNodes;
    c->dX = dalloc<double>(c->nDof, &st);
    if (!c->dX) return st;
    EF_CUDA(cudaMemcpy(c->dX, c->hX.data(), sizeof(double) * c->nDof, cudaMemcpyHostToDevice));

    c->dFlags = dalloc<int>(4, &st);
    if (!c->dFlags) return st;
    {
        const float none = EF_PNEWDT_NONE;
        int hf[4] = {0, 0, 0, 0};
        memcpy(&hf[1], &none, sizeof(float));
        EF_CUDA(cudaMemcpy(c->dFlags, hf, sizeof(hf), cudaMemcpyHostToDevice));
    }

    // groups: device node maps and double-buffered SoA state
    int64_t peOff = 0, keOff = 0, nEl = 0, nVIJ = 0;
    for (size_t gi = 0; gi < c->hg.size(); ++gi) {
        const HostGroup& h = c->hg[gi];
        Group g;
        memset(&g, 0, sizeof(g));
        g.nEl = h.nEl;
        g.nNodes = h.nNodes;
        g.nQP = h.nQP;
        g.nDofEl = 3 * h.nNodes;
        g.nPair = h.nNodes * (h.nNodes + 1) / 2;
        g.mat = h.mat;
        g.tl = h.tl;
        // FP64 <-> FP32-pair conversions by integer operations (off the FP64 pipe; the element pass
        // 0.62 -> 0.54 ms at 160k hex8 J2 elements, same results to the fixtures' tolerances);
        // EF_ELEM_INTCONV=0 uses the FP64 conversion instructions
        g.intConv = 1;
        if (const char* e = getenv("EF_ELEM_INTCONV")) g.intConv = atoi(e) != 0;
        g.cutback = (float)h.cutback;
        g.nState = 12 + ((h.mat == MAT_VON_MISES || h.mat == MAT_NEOHOOKE_WA) ? 1 : 0);
        for (size_t i = 0; i < h.props.size() && i < 8; ++i) g.props[i] = h.props[i];
        derived_props(h.mat, g.props);
        g.nodeDof = dalloc<int32_t>(h.nodeDof.size(), &st);
        if (!g.nodeDof) return st;
        EF_CUDA(cudaMemcpy(g.nodeDof, h.nodeDof.data(), sizeof(int32_t) * h.nodeDof.size(), cudaMemcpyHostToDevice));
        const size_t ns = (size_t)g.nState * h.nEl * h.nQP;
        for (int k = 0; k < 2; ++k) {
            g.state[k] = dalloc<double>(ns, &st);
            if (!g.state[k]) return st;
            EF_CUDA(cudaMemset(g.state[k], 0, sizeof(double) * ns));
        }
        g.cur = 0;
        if (!h.propsTable.empty()) {
            double* pt = dalloc<double>(h.propsTable.size(), &st);
            int32_t* er = dalloc<int32_t>(h.elemRow.size(), &st);
            if (!pt || !er) return st;
            EF_CUDA(cudaMemcpy(pt, h.propsTable.data(), sizeof(double) * h.propsTable.size(), cudaMemcpyHostToDevice));
            EF_CUDA(cudaMemcpy(er, h.elemRow.data(), sizeof(int32_t) * h.elemRow.size(), cudaMemcpyHostToDevice));
            g.propsTable = pt;
            g.elemRow = er;
        }
        g.geo = dalloc<double>((size_t)h.nEl * h.nQP * (3 * h.nNodes + 1), &st);
        if (!g.geo) return st;
        if (!g.tl) {
            g.geoS = dalloc<float2>((size_t)h.nEl * h.nQP * (3 * h.nNodes + 1), &st);
            if (!g.geoS) return st;
        }
        EF_CHECK(ef_launch_geometry(g, c->dTables[gi], c->dX, c->dFlags, 0));
        g.peOffset = peOff;
        g.keOffset = keOff;
        g.tablesSlot = (int)gi;
        peOff += (int64_t)h.nEl * g.nDofEl;
        keOff += (int64_t)h.nEl * g.nPair;
        nEl += h.nEl;
        nVIJ += (int64_t)h.nEl * g.nDofEl * g.nDofEl;
        c->groups.push_back(g);
    }
    c->nElements = nEl;
    c->nPe = peOff;
    c->nKblk = keOff;
    c->nVIJ = nVIJ;
    c->Pe = dalloc<double>(peOff, &st);
    if (!c->Pe) return st;
    c->Kblk = dalloc<char>((size_t)keOff * 9 * ks, &st);
    if (!c->Kblk) return st;

    // node -> first DOF
    std::vector<int32_t> nodeDof(nNodes);
    for (int64_t m = 0; m < nNodes; ++m) nodeDof[m] = (int32_t)(3 * m);
    c->dNodeDof = dalloc<int32_t>(nNodes, &st);
    if (!c->dNodeDof) return st;
    EF_CUDA(cudaMemcpy(c->dNodeDof, nodeDof.data(), sizeof(int32_t) * nNodes, cudaMemcpyHostToDevice));

    // ties: every node maps to target nodes with weights (itself with 1; a tied node to its two
    // masters with 1/2 each)
    const bool ties = !c->hTieS.empty();
    std::vector<int32_t> tieOf(nNodes, -1);
    for (size_t i = 0; i < c->hTieS.size(); ++i) tieOf[c->hTieS[i]] = (int32_t)i;
    auto targets = [&](int64_t m, int64_t* t, float* w) -> int {
        const int32_t k = tieOf[m];
        if (k < 0) {
            t[0] = m;
            w[0] = 1.f;
            return 1;
        }
        t[0] = c->hTieA[k];
        t[1] = c->hTieB[k];
        w[0] = w[1] = 0.5f;
        return 2;
    };
    if (ties) {
        const int64_t nt = (int64_t)c->hTieS.size();
        c->dTieS = dalloc<int32_t>(nt, &st);
        c->dTieA = dalloc<int32_t>(nt, &st);
        c->dTieB = dalloc<int32_t>(nt, &st);
        c->dTieTmp = dalloc<double>(c->nDof, &st);
        if (st != EF_OK) return st;
        EF_CUDA(cudaMemcpy(c->dTieS, c->hTieS.data(), sizeof(int32_t) * nt, cudaMemcpyHostToDevice));
        EF_CUDA(cudaMemcpy(c->dTieA, c->hTieA.data(), sizeof(int32_t) * nt, cudaMemcpyHostToDevice));
        EF_CUDA(cudaMemcpy(c->dTieB, c->hTieB.data(), sizeof(int32_t) * nt, cudaMemcpyHostToDevice));
    }

    // condensation map: node m <- Pe slices of (group, element, local node) in element order
    // (with ties: the slices of the nodes tied to m, weighted; a tied node itself gets none)
    std::vector<int64_t> cptr(nNodes + 1, 0);
    for (const auto& h : c->hg)
        for (int32_t d : h.nodeDof) {
            int64_t t[2];
            float w[2];
            const int nt = targets(d / 3, t, w);
            for (int i = 0; i < nt; ++i) cptr[t[i] + 1]++;
        }
    for (int64_t m = 0; m < nNodes; ++m) cptr[m + 1] += cptr[m];
    std::vector<int64_t> csrc(cptr[nNodes]);
    std::vector<float> cw(ties ? cptr[nNodes] : 0);
    {
        std::vector<int64_t> fill(cptr.begin(), cptr.end() - 1);
        for (size_t gi = 0; gi < c->hg.size(); ++gi) {
            const auto& h = c->hg[gi];
            const Group& g = c->groups[gi];
            for (int64_t e = 0; e < h.nEl; ++e)
                for (int a = 0; a < h.nNodes; ++a) {
                    int64_t t[2];
                    float w[2];
                    const int nt = targets(h.nodeDof[e * h.nNodes + a] / 3, t, w);
                    for (int i = 0; i < nt; ++i) {
                        const int64_t pos = fill[t[i]]++;
                        csrc[pos] = g.peOffset + e * g.nDofEl + 3 * a;
                        if (ties) cw[pos] = w[i];
                    }
                }
        }
    }
    c->dCondPtr = dalloc<int64_t>(nNodes + 1, &st);
    c->dCondSrc = dalloc<int64_t>(csrc.size(), &st);
    if (!c->dCondPtr || !c->dCondSrc) return st;
    EF_CUDA(cudaMemcpy(c->dCondPtr, cptr.data(), sizeof(int64_t) * (nNodes + 1), cudaMemcpyHostToDevice));
    EF_CUDA(cudaMemcpy(c->dCondSrc, csrc.data(), sizeof(int64_t) * csrc.size(), cudaMemcpyHostToDevice));
    if (ties) {
        c->dCondW = dalloc<float>(cw.size(), &st);
        if (!c->dCondW) return st;
        EF_CUDA(cudaMemcpy(c->dCondW, cw.data(), sizeof(float) * cw.size(), cudaMemcpyHostToDevice));
    }

    // BSR pattern + block scatter map.  Global block (m, n) = sum over elements (in order) of
    // K_ab with node(a) = m, node(b) = n; stored pair p(min,max) with a transpose flag if a > b.
    {
        std::vector<int64_t> rcount(nNodes + 1, 0);
        for (const auto& h : c->hg)
            for (int64_t e = 0; e < h.nEl; ++e) {
                int nb = 0;  // element nodes counted with their targets
                for (int b = 0; b < h.nNodes; ++b) nb += tieOf[h.nodeDof[e * h.nNodes + b] / 3] < 0 ? 1 : 2;
                for (int a = 0; a < h.nNodes; ++a) {
                    int64_t t[2];
                    float w[2];
                    const int nt = targets(h.nodeDof[e * h.nNodes + a] / 3, t, w);
                    for (int i = 0; i < nt; ++i) rcount[t[i] + 1] += nb;
                }
            }
        for (int64_t m = 0; m < nNodes; ++m)
            if (tieOf[m] >= 0) rcount[m + 1] += 1;  // the tied node's own (empty) diagonal block
        for (int64_t m = 0; m < nNodes; ++m) rcount[m + 1] += rcount[m];
        const int64_t nEnt = rcount[nNodes];
        // entries per row: (col node, element-block code); element order is preserved by the fill order
        std::vector<int32_t> ecol(nEnt);
        std::vector<int64_t> esrc(nEnt);
        std::vector<float> ew(ties ? nEnt : 0);
        std::vector<int64_t> fill(rcount.begin(), rcount.end() - 1);
        for (size_t gi = 0; gi < c->hg.size(); ++gi) {
            const auto& h = c->hg[gi];
            const Group& g = c->groups[gi];
            const int nn = h.nNodes;
            for (int64_t e = 0; e < h.nEl; ++e)
                for (int a = 0; a < nn; ++a) {
                    int64_t ta[2], tb[2];
                    float wa[2], wb[2];
                    const int na = targets(h.nodeDof[e * nn + a] / 3, ta, wa);
                    for (int ia = 0; ia < na; ++ia)
                        for (int b = 0; b < nn; ++b) {
                            const int nb = targets(h.nodeDof[e * nn + b] / 3, tb, wb);
                            const int lo = std::min(a, b), hi = std::max(a, b);
                            const int p = lo * nn - lo * (lo - 1) / 2 + (hi - lo);
                            const int64_t blk = g.keOffset + e * g.nPair + p;
                            for (int ib = 0; ib < nb; ++ib) {
                                const int64_t pos = fill[ta[ia]]++;
                                ecol[pos] = (int32_t)tb[ib];
                                esrc[pos] = (blk << 1) | (a > b ? 1 : 0);
                                if (ties) ew[pos] = wa[ia] * wb[ib];
                            }
                        }
                }
        }
        for (int64_t m = 0; m < nNodes; ++m)
            if (tieOf[m] >= 0) {  // marker of the tied node's diagonal block: no source
                const int64_t pos = fill[m]++;
                ecol[pos] = (int32_t)m;
                esrc[pos] = -1;
            }
        // per row: stable sort by column, unique columns -> blocks
        std::vector<int64_t> rowBlocks(nNodes + 1, 0);
        std::vector<int64_t> order(nEnt);
        parallel_for(nNodes, [&](int64_t lo, int64_t hi) {
            for (int64_t m = lo; m < hi; ++m) {
                const int64_t s = rcount[m], e = rcount[m + 1];
                for (int64_t i = s; i < e; ++i) order[i] = i;
                std::stable_sort(order.begin() + s, order.begin() + e,
                                 [&](int64_t x, int64_t y) { return ecol[x] < ecol[y]; });
                int64_t nb = 0;
                for (int64_t i = s; i < e; ++i)
                    if (i == s || ecol[order[i]] != ecol[order[i - 1]]) ++nb;
                rowBlocks[m + 1] = nb;
            }
        });
        for (int64_t m = 0; m < nNodes; ++m) rowBlocks[m + 1] += rowBlocks[m];
        const int64_t nBlocks = rowBlocks[nNodes];
        if (nBlocks >= ((int64_t)1 << 31)) {
            ef_set_error("ef_finalize: too many blocks");
            return EF_ERR_ARG;
        }
        c->nBlocks = nBlocks;
        std::vector<int32_t> rowPtr(nNodes + 1), colIdx(nBlocks);
        std::vector<int64_t> seg(nBlocks + 1), src(nEnt), diag(nNodes, -1);
        std::vector<float> sw(ties ? nEnt : 0);
        for (int64_t m = 0; m <= nNodes; ++m) rowPtr[m] = (int32_t)rowBlocks[m];
        parallel_for(nNodes, [&](int64_t lo, int64_t hi) {
            for (int64_t m = lo; m < hi; ++m) {
                int64_t b = rowBlocks[m] - 1;
                for (int64_t i = rcount[m]; i < rcount[m + 1]; ++i) {
                    const int64_t o = order[i];
                    if (i == rcount[m] || ecol[o] != ecol[order[i - 1]]) {
                        ++b;
                        colIdx[b] = ecol[o];
                        seg[b] = i;
                        if (ecol[o] == m) diag[m] = b;
                    }
                    src[i] = esrc[o];
                    if (ties) sw[i] = ew[o];
                }
            }
        });
        seg[nBlocks] = nEnt;
        if (ties) {
            // drop the markers of tied nodes' diagonal blocks (those blocks have no source: zero)
            std::vector<int64_t> seg2(nBlocks + 1);
            std::vector<int64_t> src2;
            std::vector<float> sw2;
            src2.reserve(nEnt);
            sw2.reserve(nEnt);
            for (int64_t b = 0; b < nBlocks; ++b) {
                seg2[b] = (int64_t)src2.size();
                for (int64_t i = seg[b]; i < seg[b + 1]; ++i)
                    if (src[i] >= 0) {
                        src2.push_back(src[i]);
                        sw2.push_back(sw[i]);
                    }
            }
            seg2[nBlocks] = (int64_t)src2.size();
            seg.swap(seg2);
            src.swap(src2);
            sw.swap(sw2);
        }
        const int64_t nSrc = (int64_t)src.size();
        for (int64_t m = 0; m < nNodes; ++m)
            if (diag[m] < 0) {
                ef_set_error("ef_finalize: a DOF triplet belongs to no element (no diagonal block)");
                return EF_ERR_ARG;
            }
        c->dRowPtr = dalloc<int32_t>(nNodes + 1, &st);
        c->dColIdx = dalloc<int32_t>(nBlocks + 16, &st);  // padding: staged loads round the end up to 16 bytes
        c->dBsrSeg = dalloc<int64_t>(nBlocks + 1, &st);
        c->dBsrSrc = dalloc<int64_t>(nSrc, &st);
        c->dDiagPos = dalloc<int64_t>(nNodes, &st);
        c->dBsrVals = dalloc<char>((size_t)nBlocks * 9 * ks + 64, &st);  // + padding for staged loads
        c->dBinv = dalloc<char>((size_t)nNodes * 9 * ks, &st);
        c->dMask = dalloc<uint8_t>(c->nDof, &st);
        if (!c->dRowPtr || !c->dColIdx || !c->dBsrSeg || !c->dBsrSrc || !c->dDiagPos || !c->dBsrVals || !c->dBinv ||
            !c->dMask)
            return st;
        EF_CUDA(cudaMemcpy(c->dRowPtr, rowPtr.data(), sizeof(int32_t) * (nNodes + 1), cudaMemcpyHostToDevice));
        EF_CUDA(cudaMemcpy(c->dColIdx, colIdx.data(), sizeof(int32_t) * nBlocks, cudaMemcpyHostToDevice));
        EF_CUDA(cudaMemcpy(c->dBsrSeg, seg.data(), sizeof(int64_t) * (nBlocks + 1), cudaMemcpyHostToDevice));
        EF_CUDA(cudaMemcpy(c->dBsrSrc, src.data(), sizeof(int64_t) * nSrc, cudaMemcpyHostToDevice));
        if (ties) {
            c->dBsrW = dalloc<float>(nSrc, &st);
            if (!c->dBsrW) return st;
            EF_CUDA(cudaMemcpy(c->dBsrW, sw.data(), sizeof(float) * nSrc, cudaMemcpyHostToDevice));
        }
        EF_CUDA(cudaMemcpy(c->dDiagPos, diag.data(), sizeof(int64_t) * nNodes, cudaMemcpyHostToDevice));
        c->hMask.assign(c->nDof, 0);
        for (int32_t sN : c->hTieS)
            for (int k = 0; k < 3; ++k) c->hMask[3 * (int64_t)sN + k] = 1;  // tied DOFs are eliminated
        EF_CUDA(cudaMemcpy(c->dMask, c->hMask.data(), c->nDof, cudaMemcpyHostToDevice));
        c->hRowPtr0 = rowPtr;
        c->hColIdx0 = colIdx;
    }

    // scalar CSR of the reference (SciPy canonical pattern) + reference-order scatter map
    if (c->scalar) {
        if (c->nVIJ >= ((int64_t)1 << 31)) {
            ef_set_error("ef_finalize: VIJ too long for the scalar CSR map; use EF_OPT_NO_SCALAR_CSR");
            return EF_ERR_ARG;
        }
        // per DOF row r: (element, local index i) occurrences in element order
        const int64_t nDof = c->nDof;
        std::vector<int64_t> rptr(nDof + 1, 0);
        for (const auto& h : c->hg)
            for (int64_t e = 0; e < h.nEl; ++e)
                for (int a = 0; a < h.nNodes; ++a)
                    for (int k = 0; k < 3; ++k) rptr[h.nodeDof[e * h.nNodes + a] + k + 1] += 3 * h.nNodes;
        for (int64_t r = 0; r < nDof; ++r) rptr[r + 1] += rptr[r];
        const int64_t nEnt = rptr[nDof];
        std::vector<int32_t> col(nEnt);
        std::vector<int32_t> kk(nEnt);
        std::vector<int64_t> fill(rptr.begin(), rptr.end() - 1);
        int64_t vijOff = 0;
        for (size_t gi = 0; gi < c->hg.size(); ++gi) {
            const auto& h = c->hg[gi];
            const int nd = 3 * h.nNodes;
            for (int64_t e = 0; e < h.nEl; ++e) {
                const int32_t* nd0 = &h.nodeDof[e * h.nNodes];
                for (int i = 0; i < nd; ++i) {
                    const int64_t r = nd0[i / 3] + i % 3;  // VIJ value p = i + j*nd -> (row d[i], col d[j])
                    for (int j = 0; j < nd; ++j) {
                        const int64_t pos = fill[r]++;
                        col[pos] = nd0[j / 3] + j % 3;
                        kk[pos] = (int32_t)(vijOff + e * (int64_t)nd * nd + i + (int64_t)j * nd);
                    }
                }
            }
            vijOff += (int64_t)h.nEl * nd * nd;
        }
        std::vector<int64_t> rowNnz(nDof + 1, 0);
        parallel_for(nDof, [&](int64_t lo, int64_t hi) {
            std::vector<std::pair<int32_t, int32_t>> tmp;
            for (int64_t r = lo; r < hi; ++r) {
                const int64_t s = rptr[r], e = rptr[r + 1];
                tmp.resize(e - s);
                for (int64_t i = s; i < e; ++i) tmp[i - s] = {col[i], kk[i]};
                std::sort(tmp.begin(), tmp.end());
                int64_t nb = 0;
                for (int64_t i = s; i < e; ++i) {
                    col[i] = tmp[i - s].first;
                    kk[i] = tmp[i - s].second;
                    if (i == s || col[i] != col[i - 1]) ++nb;
                }
                rowNnz[r + 1] = nb;
            }
        });
        for (int64_t r = 0; r < nDof; ++r) rowNnz[r + 1] += rowNnz[r];
        const int64_t nnz = rowNnz[nDof];
        c->nnz = nnz;
        c->hIndptr.resize(nDof + 1);
        c->hIndices.resize(nnz);
        std::vector<int64_t> seg(nnz + 1);
        for (int64_t r = 0; r <= nDof; ++r) c->hIndptr[r] = (int32_t)rowNnz[r];
        parallel_for(nDof, [&](int64_t lo, int64_t hi) {
            for (int64_t r = lo; r < hi; ++r) {
                int64_t sl = rowNnz[r] - 1;
                for (int64_t i = rptr[r]; i < rptr[r + 1]; ++i) {
                    if (i == rptr[r] || col[i] != col[i - 1]) {
                        ++sl;
                        c->hIndices[sl] = col[i];
                        seg[sl] = i;
                    }
                }
            }
        });
        seg[nnz] = nEnt;
        c->dIndptr = dalloc<int32_t>(nDof + 1, &st);
        c->dIndices = dalloc<int32_t>(nnz, &st);
        c->dCsrSeg = dalloc<int64_t>(nnz + 1, &st);
        c->dCsrPerm = dalloc<int32_t>(nEnt, &st);
        if (!c->dIndptr || !c->dIndices || !c->dCsrSeg || !c->dCsrPerm) return st;
        EF_CUDA(cudaMemcpy(c->dIndptr, c->hIndptr.data(), sizeof(int32_t) * (nDof + 1), cudaMemcpyHostToDevice));
        EF_CUDA(cudaMemcpy(c->dIndices, c->hIndices.data(), sizeof(int32_t) * nnz, cudaMemcpyHostToDevice));
        EF_CUDA(cudaMemcpy(c->dCsrSeg, seg.data(), sizeof(int64_t) * (nnz + 1), cudaMemcpyHostToDevice));
        EF_CUDA(cudaMemcpy(c->dCsrPerm, kk.data(), sizeof(int32_t) * nEnt, cudaMemcpyHostToDevice));
    }

    // reduction and Krylov workspaces
    c->nPart = 2 * c->nSM;
    c->dPart = dalloc<double>(4 * c->nPart, &st);
    c->dRed = dalloc<double>(16, &st);
    if (!c->dPart || !c->dRed) return st;
    EF_CHECK(ef_pcg_grid(0, c->nSM, &c->pcgGrid[0]));
    EF_CHECK(ef_pcg_grid(1, c->nSM, &c->pcgGrid[1]));
    const int maxGrid = std::max(c->pcgGrid[0], c->pcgGrid[1]);
    c->dPartA = dalloc<double>(4 * (size_t)maxGrid, &st);
    c->dPartB = dalloc<double>(4 * (size_t)maxGrid, &st);
    c->dBar = dalloc<char>(ef_barrier_state_bytes(), &st);
    c->dPcgRes = dalloc<char>(ef_pcg_result_bytes(), &st);
    if (!c->dPartA || !c->dPartB || !c->dBar || !c->dPcgRes) return st;
    EF_CUDA(cudaMemset(c->dBar, 0, ef_barrier_state_bytes()));
    for (int i = 0; i < 7; ++i) {
        c->w32[i] = dalloc<float>(c->nDof, &st);
        if (!c->w32[i]) return st;
    }
    for (int i = 0; i < 5; ++i) {
        c->w64[i] = dalloc<double>(c->nDof, &st);
        if (!c->w64[i]) return st;
    }
    if (!c->keFp64) {
        // FP32 system: keep the FP64 tangent for a matrix-free refinement residual
        for (const auto& g : c->groups) {
            const size_t nt = (size_t)(g.tl ? ef_tl_tangent_size() : 9) * g.nEl * g.nQP;
            double* t = dalloc<double>(nt, &st);
            if (!t) return st;
            EF_CUDA(cudaMemset(t, 0, sizeof(double) * nt));
            c->dTang.push_back(t);
        }
        c->dYe = dalloc<double>(c->nPe, &st);
        if (!c->dYe) return st;
        c->exact = true;
    }
    for (int i = 0; i < 7; ++i) {
        c->w64k[i] = dalloc<double>(c->nDof, &st);
        if (!c->w64k[i]) return st;
    }
    EF_CUDA(cudaEventCreate(&c->ev[0]));
    EF_CUDA(cudaEventCreate(&c->ev[1]));
    EF_CUDA(cudaEventCreate(&c->evS[0]));
    EF_CUDA(cudaEventCreate(&c->evS[1]));
    c->finalized = true;
    return EF_OK;
}

ef_status ef_get_info(const ef_ctx* c, ef_info* out) {
    if (!c || !out) return EF_ERR_ARG;
    out->nDof = c->nDof;
    out->nNodes = c->nNodes;
    out->nElements = c->nElements;
    out->nVIJ = c->nVIJ;
    out->nnz = c->nnz;
    out->nBlocks = c->nBlocks;
    out->nPe = c->nPe;
    out->keFp64 = c->keFp64;
    return EF_OK;
}



// one element pass: every group's kernel, then the condensation into P and F
static ef_status element_step(ef_ctx* c, const double* U_np, const double* dU, double* P, double* F, cudaStream_t s) {
    const size_t ks = c->keFp64 ? sizeof(double) : sizeof(float);
    for (size_t gi = 0; gi < c->groups.size(); ++gi) {
        const Group& g = c->groups[gi];
        void* K = (char*)c->Kblk + (size_t)g.keOffset * 9 * ks;
        double* tang = c->exact ? c->dTang[gi] : nullptr;
        if (g.tl)
            EF_CHECK(ef_launch_total_lagrange(g, U_np, K, c->keFp64, 0, c->Pe + g.peOffset, tang, c->dFlags, s));
        else
            EF_CHECK(ef_launch_small_strain(g, dU, K, c->keFp64, 0, c->Pe + g.peOffset, tang, c->dFlags, s));
    }
    EF_CHECK(ef_launch_condense(c->nNodes, c->dNodeDof, c->dCondPtr, c->dCondSrc, c->dCondW, c->Pe, P, F, s));
    return EF_OK;
}


// With several element groups (element types), the pass is captured as one CUDA graph the second
// time it runs on the same vectors and replayed from then on.
ef_status ef_compute_elements(ef_ctx* c, const double* U_np, const double* dU, const double* time2, double dT,
                              double* P, double* F, void* stream) {
    EF_REQUIRE_FINALIZED(c);
    (void)time2;
    (void)dT;
    if (!dU || !P) {
        ef_set_error("ef_compute_elements: null vector");
        return EF_ERR_ARG;
    }
    for (const auto& g : c->groups)
        if (g.tl && !U_np) {
            ef_set_error("ef_compute_elements: total-Lagrange elements need U_np");
            return EF_ERR_ARG;
        }
    cudaStream_t s = (cudaStream_t)stream;
    if (c->groups.size() < 2 || !c->elemGraphs) return element_step(c, U_np, dU, P, F, s);
    const void* key[4] = {U_np, dU, P, F};
    const bool same = memcmp(key, c->egKey, sizeof(key)) == 0;
    if (same && c->egExec) {
        ef::note_launches(c->egKernels);
        EF_CUDA(cudaGraphLaunch(c->egExec, s));
        return EF_OK;
    }
    if (!same) {  // new vectors: run eagerly and remember them
        if (c->egExec) cudaGraphExecDestroy(c->egExec);
        c->egExec = nullptr;
        memcpy(c->egKey, key, sizeof(key));
        return element_step(c, U_np, dU, P, F, s);
    }
    if (!c->capStream) EF_CUDA(cudaStreamCreateWithFlags(&c->capStream, cudaStreamNonBlocking));
    EF_CUDA(cudaStreamBeginCapture(c->capStream, cudaStreamCaptureModeThreadLocal));
    long long captured = 0;
    t_captureCount = &captured;
    const ef_status st = element_step(c, U_np, dU, P, F, c->capStream);
    t_captureCount = nullptr;
    cudaGraph_t g = nullptr;
    const cudaError_t e = cudaStreamEndCapture(c->capStream, &g);
    if (st != EF_OK) return st;
    if (e != cudaSuccess) {
        ef_set_error(std::string("element-pass capture: ") + cudaGetErrorString(e));
        return EF_ERR_CUDA;
    }
    EF_CUDA(cudaGraphInstantiate(&c->egExec, g, 0));
    cudaGraphDestroy(g);
    c->egKernels = captured;
    ef::note_launches(c->egKernels);
    EF_CUDA(cudaGraphLaunch(c->egExec, s));
    return EF_OK;
}

ef_status ef_element_status(ef_ctx* c, void* stream, double* pNewDT) {
    EF_REQUIRE_FINALIZED(c);
    int hf[2] = {0, 0};
    EF_CUDA(cudaMemcpyAsync(hf, c->dFlags, sizeof(hf), cudaMemcpyDeviceToHost, (cudaStream_t)stream));
    EF_CUDA(cudaStreamSynchronize((cudaStream_t)stream));
    const int f = hf[0];
    float req = EF_PNEWDT_NONE;
    memcpy(&req, &hf[1], sizeof(float));
    {
        const float none = EF_PNEWDT_NONE;
        int reset[2] = {0, 0};
        memcpy(&reset[1], &none, sizeof(float));
        EF_CUDA(cudaMemcpy(c->dFlags, reset, sizeof(reset), cudaMemcpyHostToDevice));
    }
    if (pNewDT) *pNewDT = 1.0;
    if (f & EF_FLAG_NAN) return EF_NAN;
    if (f & EF_FLAG_RETURNMAP) {
        // the smallest scale any failing element asked for (min over elements, as the Marmot
        // element loop's min over its threads' pNewDT, solvers/nonlinearimplicitstaticparallel.pyx:145-150)
        if (pNewDT) *pNewDT = req < EF_PNEWDT_NONE ? (double)req : 0.5;
        return EF_CUTBACK;
    }
    if (f & EF_FLAG_BADDET) {
        ef_set_error("non-positive Jacobian determinant in an element");
        return EF_ERR_DEVICE;
    }
    if (f & EF_FLAG_BARRIER) {
        ef_set_error("a device-side grid barrier timed out");
        return EF_ERR_DEVICE;
    }
    return EF_OK;
}

ef_status ef_get_state_size(const ef_ctx* c, int groupId, int* nQP, int* nState) {
    if (!c || !c->finalized || groupId < 0 || groupId >= (int)c->groups.size()) return EF_ERR_ARG;
    if (nQP) *nQP = c->groups[groupId].nQP;
    if (nState) *nState = c->groups[groupId].nState;
    return EF_OK;
}

// host AoS [nEl][nQP][nState] <-> device SoA [nState][nEl*nQP]
ef_status ef_set_state(ef_ctx* c, int groupId, const double* state) {
    EF_REQUIRE_FINALIZED(c);
    if (groupId < 0 || groupId >= (int)c->groups.size() || !state) return EF_ERR_ARG;
    const Group& g = c->groups[groupId];
    const int64_t nq = (int64_t)g.nEl * g.nQP;
    std::vector<double> soa((size_t)nq * g.nState);
    for (int64_t i = 0; i < nq; ++i)
        for (int v = 0; v < g.nState; ++v) soa[v * nq + i] = state[i * g.nState + v];
    EF_CUDA(cudaMemcpy(g.state[g.cur], soa.data(), sizeof(double) * soa.size(), cudaMemcpyHostToDevice));
    return EF_OK;
}

ef_status ef_get_state(ef_ctx* c, int groupId, int trial, double* state) {
    EF_REQUIRE_FINALIZED(c);
    if (groupId < 0 || groupId >= (int)c->groups.size() || !state) return EF_ERR_ARG;
    const Group& g = c->groups[groupId];
    const int64_t nq = (int64_t)g.nEl * g.nQP;
    std::vector<double> soa((size_t)nq * g.nState);
    EF_CUDA(cudaDeviceSynchronize());
    EF_CUDA(cudaMemcpy(soa.data(), g.state[trial ? 1 - g.cur : g.cur], sizeof(double) * soa.size(),
                       cudaMemcpyDeviceToHost));
    for (int64_t i = 0; i < nq; ++i)
        for (int v = 0; v < g.nState; ++v) state[i * g.nState + v] = soa[v * nq + i];
    return EF_OK;
}

ef_status ef_accept_state(ef_ctx* c) {
    EF_REQUIRE_FINALIZED(c);
    // copy trial -> committed (acceptLastState copies stateTemp into stateRef); the buffers keep
    // their roles, so launches captured in CUDA graphs stay valid across increments
    for (auto& g : c->groups)
        EF_CUDA(cudaMemcpy(g.state[g.cur], g.state[1 - g.cur], sizeof(double) * g.nState * g.nEl * g.nQP,
                           cudaMemcpyDeviceToDevice));
    return EF_OK;
}

ef_status ef_reset_state(ef_ctx* c) {
    EF_REQUIRE_FINALIZED(c);
    for (auto& g : c->groups)
        EF_CUDA(cudaMemcpy(g.state[1 - g.cur], g.state[g.cur], sizeof(double) * g.nState * g.nEl * g.nQP,
                           cudaMemcpyDeviceToDevice));
    return EF_OK;
}

ef_status ef_add_body_force(ef_ctx* c, int groupId, const double* load3, double* PExt, void* stream) {
    EF_REQUIRE_FINALIZED(c);
    if (groupId < 0 || groupId >= (int)c->groups.size() || !load3 || !PExt) {
        ef_set_error("ef_add_body_force: invalid arguments");
        return EF_ERR_ARG;
    }
    const Group& g = c->groups[groupId];
    cudaStream_t s = (cudaStream_t)stream;
    EF_CHECK(ef_launch_body_force(g, c->dTables[groupId], load3, c->Pe + g.peOffset, s));
    EF_CHECK(ef_launch_condense_add(c->nNodes, c->dNodeDof, c->dCondPtr, c->dCondSrc, c->dCondW, c->Pe, g.peOffset,
                                    g.peOffset + (int64_t)g.nEl * g.nDofEl, PExt, s));
    return EF_OK;
}

// ---- element result collectors (utils/elementresultcollector.pyx:38-120) ----------------------

static ResultCollector* result_collector(ef_ctx* c, int id) {
    if (id < 0 || id >= (int)c->results.size() || c->results[id].group < 0) {
        ef_set_error("element result collector: unknown id");
        return nullptr;
    }
    return &c->results[id];
}

ef_status ef_results_create(ef_ctx* c, int groupId, const int32_t* elements, int nEls, const int32_t* qps, int nQps,
                            int first, int count, int* collectorId) {
    EF_REQUIRE_FINALIZED(c);
    if (groupId < 0 || groupId >= (int)c->groups.size() || !collectorId) {
        ef_set_error("ef_results_create: invalid group or output");
        return EF_ERR_ARG;
    }
    const Group& g = c->groups[groupId];
    if (first < 0 || count < 1 || first + count > g.nState) {
        ef_set_error("ef_results_create: state slice outside [0, nState)");
        return EF_ERR_ARG;
    }
    std::vector<int32_t> el, qp;
    if (elements) {
        if (nEls < 1) {
            ef_set_error("ef_results_create: empty element list");
            return EF_ERR_ARG;
        }
        el.assign(elements, elements + nEls);
    } else {
        el.resize(g.nEl);
        for (int e = 0; e < g.nEl; ++e) el[e] = e;
    }
    if (qps) {
        if (nQps < 1) {
            ef_set_error("ef_results_create: empty quadrature point list");
            return EF_ERR_ARG;
        }
        qp.assign(qps, qps + nQps);
    } else {
        qp.resize(g.nQP);
        for (int q = 0; q < g.nQP; ++q) qp[q] = q;
    }
    for (int32_t e : el)
        if (e < 0 || e >= g.nEl) {
            ef_set_error("ef_results_create: element index outside the group");
            return EF_ERR_ARG;
        }
    for (int32_t q : qp)
        if (q < 0 || q >= g.nQP) {
            ef_set_error("ef_results_create: quadrature point outside the element");
            return EF_ERR_ARG;
        }
    ResultCollector r;
    r.nEls = (int)el.size();
    r.nQ = (int)qp.size();
    r.first = first;
    r.count = count;
    ef_status st = upload(&r.dEl, el);
    if (st == EF_OK) st = upload(&r.dQp, qp);
    if (st == EF_OK) r.dTable = dalloc<double>((size_t)r.nEls * r.nQ * count, &st);
    if (st != EF_OK) {
        for (void* p : {(void*)r.dEl, (void*)r.dQp, (void*)r.dTable})
            if (p) cudaFree(p);
        return st;
    }
    r.group = groupId;
    int id = 0;
    while (id < (int)c->results.size() && c->results[id].group >= 0) ++id;
    if (id == (int)c->results.size())
        c->results.push_back(r);
    else
        c->results[id] = r;
    *collectorId = id;
    return EF_OK;
}

ef_status ef_results_update(ef_ctx* c, int collectorId, int trial, double* hostOut, void* stream) {
    EF_REQUIRE_FINALIZED(c);
    const ResultCollector* r = result_collector(c, collectorId);
    if (!r) return EF_ERR_ARG;
    const Group& g = c->groups[r->group];
    cudaStream_t s = (cudaStream_t)stream;
    const int64_t nPts = (int64_t)r->nEls * r->nQ;
    EF_CHECK(ef_launch_results_gather(nPts, r->nQ, g.nQP, (int64_t)g.nEl * g.nQP, r->first, r->count, r->dEl, r->dQp,
                                      g.state[trial ? 1 - g.cur : g.cur], r->dTable, s));
    if (hostOut) {
        EF_CUDA(cudaMemcpyAsync(hostOut, r->dTable, sizeof(double) * nPts * r->count, cudaMemcpyDeviceToHost, s));
        EF_CUDA(cudaStreamSynchronize(s));
    }
    return EF_OK;
}

ef_status ef_results_device(ef_ctx* c, int collectorId, const double** table, int64_t* nValues) {
    EF_REQUIRE_FINALIZED(c);
    const ResultCollector* r = result_collector(c, collectorId);
    if (!r || !table) return EF_ERR_ARG;
    *table = r->dTable;
    if (nValues) *nValues = (int64_t)r->nEls * r->nQ * r->count;
    return EF_OK;
}

ef_status ef_results_destroy(ef_ctx* c, int collectorId) {
    EF_REQUIRE_FINALIZED(c);
    ResultCollector* r = result_collector(c, collectorId);
    if (!r) return EF_ERR_ARG;
    EF_CUDA(cudaFree(r->dEl));
    EF_CUDA(cudaFree(r->dQp));
    EF_CUDA(cudaFree(r->dTable));
    *r = ResultCollector();
    return EF_OK;
}

