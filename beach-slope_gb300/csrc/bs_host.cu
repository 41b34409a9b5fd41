// bs_host.cu -- the C-ABI (include/beachslope.h): context lifetime, upload /
// download, one entry point per reference subroutine and the fused step.
#include <cuda_runtime.h>

#include <algorithm>
#include <array>
#include <atomic>
#include <cmath>
#include <cstdio>
#include <cstddef>
#include <cstring>
#include <string>
#include <thread>
#include <vector>

#include "bs_internal.cuh"

namespace bs {
void projection_only(const Dev& D, const Launch& L);
void disp(const Dev& D, const Launch& L);
void velmag(const Dev& D, const Launch& L);
}  // namespace bs

struct bs_ctx {
    int nscene = 0;
    std::vector<bs_params> prm;
    std::vector<ScenePar> hpar;
    int nrow_total = 0, nblk_total = 0, ncell_total = 0, kmax = 0, ngrain_total = 0, ngrp_total = 0;
    int precision = 0;
    std::vector<int> grain0, gcap;
    Dev D{};
    cudaStream_t stream = nullptr;
    cudaEvent_t ev[16] = {};
    cudaEvent_t evsync = nullptr;
    int64_t launches = 0;
    std::string err;
    int* h_pinned = nullptr;   // [0] converged counter, [1..] solsteps per scene
    int* d_nconv = nullptr;
    std::vector<void*> allocs;
    std::vector<size_t> alloc_bytes;   // size of each entry of allocs
    bool assembled = false;
    bool disp_ready = false;
    int max_solsteps = 1;
    bs::KTimer timer;
    bs::IterGraph graph;
    std::vector<MgLevel> mglev;          // multigrid level tables (kernel arguments), index = level
    std::vector<std::vector<std::pair<int, int>>> mgdims;   // per scene: current grid of each level
    std::vector<std::vector<int>> mgrange;   // per scene: cells reserved on each level (fixed at create)
    std::vector<int> cellx_cap, celly_cap;   // per scene: largest cell grid the slot takes
    std::vector<unsigned char> mgneed;   // per level: which launches some scene needs (Launch::mgneed)
    // open-boundary buffer zones, per scene and zone (0, 1)
    struct Zone {
        bool set = false;
        bs::ZoneDev dev{};
        double period = 0, phase = 0;
        long next_k = 1;
        int n = 0;          // template particles inside entry cells
        double* mem = nullptr;   // x, y, vx, vy, p of the template, grouped by cell
        int* pmem = nullptr;     // pid
    };
    std::vector<std::array<Zone, 2>> zones;
    bool any_zone = false;
    std::vector<SceneDyn> hdyn;   // host copy of the scenes' dynamic state (schedule of the zones)
    // asynchronous read-back (bs_download_async): the device snapshot (per
    // field a region of nrow_total rows, then tid and pid as int32, flags,
    // the scenes' dynamic state), the copy stream and its events, the host
    // copy of each scene's dynamic state at its snapshot
    char* snap = nullptr;
    cudaStream_t cstream = nullptr;
    cudaEvent_t ev_snap = nullptr;
    std::vector<cudaEvent_t> ev_copied;   // per scene: its last copy to the host
    SceneDyn* h_snapdyn = nullptr;
    // multigrid levels run as one clustered launch per visit (mg_sub option)
    int mgsub_on = 0, mgsub_level = 0, mgsub_cs = 1, sm_count = 0;
    // the last two levels of a visit in one block per scene (option mg_tail,
    // default on: bit-identical to the separate launches): the level it
    // starts at (0: off or no level qualifies)
    int mgtail_on = 1, mgtail_level = 0;
    // FGMRES basis as double-float (hi, lo) FP32 pairs in the preconditioned mixed solve
    int fg_df_on = 1;
    // option "mg_fp32": the FP64 form's multigrid preconditioner in FP32 (the
    // mixed form's cycle; the Krylov solve and its stopping test stay FP64)
    int mg_fp32 = 0;
    // threads per block of the neighbour sweeps and of the particle-level
    // multigrid kernels (options "sweep_tpb", "mg0_tpb"; the autotuner picks them)
    int sweep_tpb = BS_THREADS, mg0_tpb = BS_THREADS;
    // exact coarse solve (option "mg_exact"): the scenes' exactly solved levels
    MgExact mgexact{};
    // captured production steps (one CUDA graph per step, loops on the device):
    // cache keyed by the bytes the capture depends on; the pointer pairs the
    // stages swap cycle with a period of a few steps, so a few entries serve
    struct StepGraph {
        cudaGraphExec_t exec = nullptr;
        std::vector<unsigned char> key;
        Dev after{};            // the device tables after the step (the swaps the capture made)
        bool disp_after = false;
        int64_t kernels = 0;    // kernels outside the device loops
        uint64_t used = 0;
    };
    std::vector<StepGraph> sgraphs;
    int step_graph_on = 1;      // option "step_graph"
    bool step_graph_broken = false;   // a capture failed: eager steps from then on
    uint64_t sg_clock = 0;
    int64_t graph_steps = 0;
    bool solsteps_stale = false;      // solsteps not read back since the last captured step
    cudaStream_t side[3] = {};        // streams that capture the loop bodies
};

namespace {

// drop the captured steps (their kernels hold the old tables and sizes)
void sg_clear(bs_ctx* ctx) {
    for (auto& g : ctx->sgraphs)
        if (g.exec) cudaGraphExecDestroy(g.exec);
    ctx->sgraphs.clear();
}

int fail(bs_ctx* c, int code, const std::string& m) {
    if (c) c->err = m;
    return code;
}

#define CK(call)                                                                             \
    do {                                                                                     \
        cudaError_t e_ = (call);                                                             \
        if (e_ != cudaSuccess) return fail(ctx, BS_E_CUDA, std::string(#call ": ") + cudaGetErrorString(e_)); \
    } while (0)

template <class T>
int dalloc(bs_ctx* ctx, T** p, size_t n) {
    void* q = nullptr;
    if (n == 0) n = 1;
    cudaError_t e = cudaMalloc(&q, n * sizeof(T));
    if (e != cudaSuccess) return fail(ctx, BS_E_NOMEM, std::string("cudaMalloc: ") + cudaGetErrorString(e));
    cudaMemset(q, 0, n * sizeof(T));
    ctx->allocs.push_back(q);
    ctx->alloc_bytes.push_back(n * sizeof(T));
    *p = (T*)q;
    return 0;
}

template <class T>
void dfree(bs_ctx* ctx, T*& p) {
    if (!p) return;
    for (size_t i = 0; i < ctx->allocs.size(); ++i)
        if (ctx->allocs[i] == (void*)p) {
            ctx->allocs.erase(ctx->allocs.begin() + i);
            ctx->alloc_bytes.erase(ctx->alloc_bytes.begin() + i);
            break;
        }
    cudaFree(p);
    p = nullptr;
}

// FGMRES storage for the context's restart length and preconditioner: basis
// V [(m+1) x rows], preconditioned basis Z [m x rows] (only with the
// multigrid cycle), block partials and the per-scene small matrices
int fg_ensure(bs_ctx* ctx) {
    Dev& D = ctx->D;
    const int m = ctx->prm[0].ppe_restart;
    const bool precond = ctx->prm[0].ppe_precond != 0;
    if (m < 1 || m > BS_FG_MAXM) return fail(ctx, BS_E_ARG, "ppe_restart outside 1..150");
    if (D.fg_V && D.fg_m == m && (!precond || D.fg_Z)) return 0;
    cudaStreamSynchronize(ctx->stream);
    auto release = [&]() {
        dfree(ctx, D.fg_V);
        dfree(ctx, D.fg_Z);
        dfree(ctx, D.fg_part);
        dfree(ctx, D.fg_gpart);
        dfree(ctx, D.fg_small);
        dfree(ctx, D.fg_gdone);
    };
    release();
    const size_t R = ctx->nrow_total;
    const size_t ld = bs::fg_part_ld(m);
    int rc = dalloc(ctx, &D.fg_V, (size_t)(m + 1) * R);
    if (!rc && precond) rc = dalloc(ctx, &D.fg_Z, (size_t)m * R);
    if (!rc) rc = dalloc(ctx, &D.fg_part, (size_t)ctx->nblk_total * ld);
    if (!rc) rc = dalloc(ctx, &D.fg_gpart, (size_t)ctx->ngrp_total * ld);
    if (!rc) rc = dalloc(ctx, &D.fg_gdone, (size_t)ctx->ngrp_total);
    if (!rc) rc = dalloc(ctx, &D.fg_small, (size_t)ctx->nscene * bs::fg_small_size(m));
    if (rc) {
        release();
        D.fg_m = 0;
        return rc;
    }
    D.fg_m = m;
    D.fg_ld = (int)R;
    D.fg_small_n = bs::fg_small_size(m);
    ctx->graph.valid = false;
    return 0;
}

// precision of the multigrid preconditioner's cycle (its setup, matrix copy and level arrays)
int mg_prec_of(const bs_ctx* c) { return (c->precision == BS_PREC_MIXED || c->mg_fp32) ? BS_PREC_MIXED : BS_PREC_FP64; }

bs::Launch launch_of(bs_ctx* c) {
    bs::Launch L;
    L.stream = c->stream;
    L.nblk_rows = c->nblk_total;
    L.ncell_total = c->ncell_total;
    L.launches = &c->launches;
    L.timer = &c->timer;
    L.graph = &c->graph;
    L.mglev = c->mglev.empty() ? nullptr : c->mglev.data();
    L.mgneed = c->mgneed.empty() ? nullptr : c->mgneed.data();
    L.mgsub_level = c->mgsub_level;
    L.mgtail = c->mgtail_level;
    L.mgsub_cs = c->mgsub_cs;
    L.sweep_tpb = c->sweep_tpb;
    L.mg0_tpb = c->mg0_tpb;
    L.exact = &c->mgexact;
    return L;
}

// multigrid grids of a scene: level 1 = half-cells, then 2x2 coarsening
// until at most 256 cells (each scene on its own, so its cycle is the same
// alone and inside any batch)
std::vector<std::pair<int, int>> mg_dims_of(int cellx, int celly) {
    std::vector<std::pair<int, int>> d;
    int nx = 2 * cellx, ny = 2 * celly;
    d.push_back({nx, ny});
    while (nx * ny > 256 && (int)d.size() < BS_MG_MAXL) {
        nx = (nx + 1) / 2;
        ny = (ny + 1) / 2;
        d.push_back({nx, ny});
    }
    return d;
}

// Operations of one visit of level l (the recursion of the cycle)
int mg_sub_nops(const bs_ctx* c, int l) {
    const unsigned char need = c->mgneed[l];
    if (!(need & 1)) return 0;
    int n = (need & 4) ? 1 : 0;
    if (!(need & 2)) return n;
    n += 2 + mg_sub_nops(c, l + 1);
    if (l <= c->D.mg.wlev) n += 1 + mg_sub_nops(c, l + 1);
    return n;
}

// First level from which the cycle runs as one clustered launch: the
// shallowest level whose largest scene fits one cluster of up to 16 blocks
// of 1024 threads (a cell per thread), all scenes' clusters fit on the SMs at
// once, the levels below fit the launch's tables and the visit's op list its
// array; 0 when there is none (or the option is off).
void mg_sub_choose(bs_ctx* c) {
    c->mgsub_level = 0;
    c->mgsub_cs = 1;
    const MgDev& M = c->D.mg;
    if (!c->mgsub_on || M.exact || c->mglev.empty() || M.nlev < 1) return;
    for (int l = 1; l <= M.nlev; ++l) {
        if (!(c->mgneed[l] & 1)) break;
        int mx = 0;
        for (int s = 0; s < c->nscene; ++s) mx = std::max(mx, c->mglev[l].nx[s] * c->mglev[l].ny[s]);
        const int cs = std::max(1, (mx + 1023) / 1024);
        if (cs > 16 || (long)cs * c->nscene > c->sm_count) continue;
        if (M.nlev - l + 1 > BS_MG_SUBL || mg_sub_nops(c, l) > BS_MG_MAXOPS) continue;
        const size_t smem = 2 * (size_t)M.coarse_max * (mg_prec_of(c) == BS_PREC_MIXED ? sizeof(float) : sizeof(double));
        if (bs::mg_sub_max_clusters(mg_prec_of(c), cs, smem) < 1) continue;
        c->mgsub_level = l;
        c->mgsub_cs = cs;
        return;
    }
}

// The level whose visits run with the coarsest level in one block per scene
// (k_mg_tail): every scene that has it has its coarsest level right below it,
// with at most 1024 cells on it and 256 on the coarsest; 0 when none does or
// the option, the exact coarse solve or the clustered subtree is on.
int coarsest_level(const bs_ctx* c, int s);
void mg_tail_choose(bs_ctx* c) {
    const MgDev& M = c->D.mg;
    c->mgtail_level = 0;
    if (!c->mgtail_on || M.exact || c->mgsub_level || c->mglev.empty()) return;
    for (int l = 1; l < M.nlev; ++l) {
        bool ok = true, any = false;
        for (int s = 0; s < c->nscene && ok; ++s) {
            if (coarsest_level(c, s) < l) continue;
            any = true;
            const int mf = c->mglev[l].nx[s] * c->mglev[l].ny[s], mc = c->mglev[l + 1].nx[s] * c->mglev[l + 1].ny[s];
            ok = coarsest_level(c, s) == l + 1 && mf <= 1024 && mc <= 256;
        }
        if (ok && any) {
            c->mgtail_level = l;
            return;
        }
    }
}

// A scene's coarsest level: where its hierarchy ends (at most 256 cells), or
// with the exact coarse solve its first level of at most BS_MG_EXACT_MAX
// cells whose band LU factors fit the factorisation's shared memory.
int coarsest_level(const bs_ctx* c, int s) {
    const auto& d = c->mgdims[s];
    if (c->D.mg.exact)
        for (int l = 1; l <= (int)d.size(); ++l) {
            const long m = (long)d[l - 1].first * d[l - 1].second;
            if (m <= BS_MG_EXACT_MAX && m * (2L * (d[l - 1].second + 1) + 1) <= BS_MG_EXACT_BAND) return l;
        }
    return (int)d.size();
}

// Level tables (kernel arguments), the launches each level needs, and the
// device copies of the current grids, from the scenes' current grids and the
// fixed per-level ranges.
void mg_tables(bs_ctx* c) {
    MgDev& M = c->D.mg;
    const int L = M.nlev, ns = c->nscene;
    c->mglev.assign(L + 2, MgLevel{});
    c->mgneed.assign(L + 2, 0);
    for (int l = 1; l <= L; ++l) {
        MgLevel& G = c->mglev[l];
        G.l = l;
        G.n = M.n[l];
        G.ns = ns;
        int o = 0;
        std::vector<int> nxv(ns, 0), nyv(ns, 0);
        for (int s = 0; s < ns; ++s) {
            G.off[s] = o;
            const int Lc = coarsest_level(c, s);
            const bool has = Lc >= l;
            G.nx[s] = nxv[s] = has ? c->mgdims[s][l - 1].first : 0;
            G.ny[s] = nyv[s] = has ? c->mgdims[s][l - 1].second : 0;
            G.lev[s] = Lc;
            o += (int)c->mgrange[s].size() >= l ? c->mgrange[s][l - 1] : 0;
            if (l <= Lc) c->mgneed[l] |= 1;
            if (l < Lc) c->mgneed[l] |= 2;
            if (l == Lc) c->mgneed[l] |= 4;
        }
        G.off[ns] = o;
        cudaMemcpy((void*)M.nx[l], nxv.data(), sizeof(int) * ns, cudaMemcpyHostToDevice);
        cudaMemcpy((void*)M.ny[l], nyv.data(), sizeof(int) * ns, cudaMemcpyHostToDevice);
    }
    c->mgexact = MgExact{};
    c->mgexact.ns = ns;
    for (int s = 0; s < ns; ++s) {
        const int Lc = coarsest_level(c, s);
        c->hpar[s].mg_lev = Lc;
        if (M.exact && Lc >= 1) {
            c->mgexact.l[s] = Lc;
            c->mgexact.off[s] = c->mglev[Lc].off[s];
            c->mgexact.nx[s] = c->mglev[Lc].nx[s];
            c->mgexact.ny[s] = c->mglev[Lc].ny[s];
        }
    }
    mg_sub_choose(c);
    mg_tail_choose(c);
}

// per-scene constants that do not depend on the layout
void fill_par(ScenePar& P, const bs_params& p, int kmax) {
    P.h = p.h; P.twoh = 2.0 * p.h; P.lam = 0.0010 * (p.h * p.h); P.dl = p.dl; P.cw = 4.0 * p.h;
    P.inv_h = 1.0 / p.h; P.inv_h2 = 1.0 / (p.h * p.h); P.inv_h3 = 1.0 / (p.h * p.h * p.h);
    P.cn1 = 0.1 * (10.0 / (BS_C28 * (p.h * p.h)));
    P.cn2 = (1.0 - 0.1) * (1.0 / (BS_C3 * (p.h * p.h)));
    P.wo = 0.1 * 4.0 * (10.0 / (BS_C28 * (p.h * p.h))) + (1.0 - 0.1) * 6.0 * (1.0 / (BS_C3 * (p.h * p.h)));
    const double kr = P.cn2 / P.cn1, k3 = 3.0 * (1.0 + kr);
    P.kq_s = (float)(P.cn1 * P.inv_h2);
    P.kq_rho_h = (float)kr;
    P.kq_rho_l = (float)(kr - (double)P.kq_rho_h);
    P.kq_k3_h = (float)k3;
    P.kq_k3_l = (float)(k3 - (double)P.kq_k3_h);
    P.kq_lam_h = (float)P.lam;
    P.kq_lam_l = (float)(P.lam - (double)P.kq_lam_h);
    P.kq_pad = 0.0f;
    P.rho = p.rho; P.rhomin = p.rhomin; P.rhomax = p.rhomax; P.rel_den = p.rel_den; P.g = p.g;
    P.mu = p.mu; P.tschmidt = p.tschmidt; P.por = p.por; P.lamk = p.lamk; P.d50 = p.d50;
    P.freethr = p.lamfs * p.maxdivr; P.csh = p.csh; P.maxshift = p.maxshift; P.sig1 = p.sig1;
    P.xlcutoff = p.xlcutoff; P.ytcutoff = p.ytcutoff; P.ppe_tol = p.ppe_tol; P.inner_tol = p.mixed_inner_tol;
    P.buf_lo = p.buf_release_lo; P.buf_hi = p.buf_release_hi;
    P.wc_c0 = p.wc_c0; P.wc_gamma = p.wc_gamma; P.wc_delta = p.wc_delta; P.wc_ysurf = p.wc_ysurf;
    P.wc_form = p.wc_form;
    P.cellx = p.cellx; P.celly = p.celly; P.ncell = p.cellx * p.celly;
    P.kmax = kmax; P.maxit = p.ppe_maxit;
    P.adaptive_dt = p.adaptive_dt; P.scalar_on = p.scalar_on; P.precision = p.precision; P.stop_rule = p.ppe_stop;
    P.max_outer = p.mixed_max_outer;
}

// cell bounds as setup.f90:120-123
double xleft_of(const bs_params& p, int j) { return (double)(j - 2) * (4.0 * p.h); }
double xright_of(const bs_params& p, int j) { return (double)(j - 1) * (4.0 * p.h); }
double ybot_of(const bs_params& p, int i) { return (double)(-i + p.celly - 1) * (4.0 * p.h); }
double ytop_of(const bs_params& p, int i) { return (double)(-i + p.celly) * (4.0 * p.h); }

bool locate(const bs_params& p, double x, double y, int* ci, int* cj) {
    if (!std::isfinite(x) || !std::isfinite(y)) return false;
    const double cw = 4.0 * p.h;
    int j = (int)std::floor(x / cw) + 2;
    j = std::max(1, std::min(p.cellx, j));
    for (int it = 0; it < 4; ++it) {
        if (x < xleft_of(p, j) && j > 1) --j;
        else if (!(x < xright_of(p, j)) && j < p.cellx) ++j;
        else break;
    }
    int i = p.celly - 1 - (int)std::floor(y / cw);
    i = std::max(1, std::min(p.celly, i));
    for (int it = 0; it < 4; ++it) {
        if (y < ybot_of(p, i) && i < p.celly) ++i;
        else if (!(y < ytop_of(p, i)) && i > 1) --i;
        else break;
    }
    if (!(x >= xleft_of(p, j) && x < xright_of(p, j) && y >= ybot_of(p, i) && y < ytop_of(p, i))) return false;
    if (i < 2 || i > p.celly - 1 || j < 2 || j > p.cellx - 1) return false;
    *ci = i;
    *cj = j;
    return true;
}

void swap_particles(Dev& D) {
    std::swap(D.x, D.x2); std::swap(D.y, D.y2); std::swap(D.xs, D.xs2); std::swap(D.ys, D.ys2);
    std::swap(D.vx, D.vx2); std::swap(D.vy, D.vy2); std::swap(D.vxs, D.vxs2); std::swap(D.vys, D.vys2);
    std::swap(D.p, D.p2); std::swap(D.mass, D.mass2); std::swap(D.rho, D.rho2); std::swap(D.oden, D.oden2);
    std::swap(D.ovol, D.ovol2); std::swap(D.con, D.con2); std::swap(D.vol, D.vol2); std::swap(D.nu, D.nu2);
    std::swap(D.tid, D.tid2); std::swap(D.flags, D.flags2); std::swap(D.pid, D.pid2); std::swap(D.cell, D.cell2);
    std::swap(D.cell_start, D.cell_start2);
    std::swap(D.cell_end, D.cell_end2);
}

int read_solsteps(bs_ctx* ctx) {
    Dev& D = ctx->D;
    CK(cudaMemcpy2DAsync(ctx->h_pinned + 1, sizeof(int), &D.dyn[0].solsteps, sizeof(SceneDyn), sizeof(int),
                         ctx->nscene, cudaMemcpyDeviceToHost, ctx->stream));
    CK(cudaStreamSynchronize(ctx->stream));
    int mx = 1;
    for (int s = 0; s < ctx->nscene; ++s) mx = std::max(mx, ctx->h_pinned[1 + s]);
    ctx->max_solsteps = mx;
    bs::timer_collect(&ctx->timer, false);
    return 0;
}

int check_launch(bs_ctx* ctx) {
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return fail(ctx, BS_E_CUDA, std::string("kernel launch: ") + cudaGetErrorString(e));
    return 0;
}

// stage helpers (no sync)
void st_rebin(bs_ctx* c, int projection, int cutoff) {
    bs::rebin(c->D, launch_of(c), projection, cutoff);
    swap_particles(c->D);
}
void st_search(bs_ctx* c, int do_search, int do_effpor) {
    bs::search(c->D, launch_of(c), c->precision, do_search, do_effpor);
    if (do_effpor) {
        std::swap(c->D.rho, c->D.rho_new);
        std::swap(c->D.vol, c->D.vol_new);
    }
}
void st_scalar(bs_ctx* c, int substep) {
    bs::scalar(c->D, launch_of(c), c->precision, substep);
    std::swap(c->D.con, c->D.con_new);
}
int st_solve(bs_ctx* c) {
    bs::Launch L = launch_of(c);
    int maxit = 0;
    for (auto& p : c->prm) maxit = std::max(maxit, (int)p.ppe_maxit);
    if (c->prm[0].ppe_solver == BS_SOLVER_FGMRES) {
        if (int rc = fg_ensure(c)) return rc;
        // the double-float basis serves the preconditioned mixed solve (the
        // basis is only read by the Gram-Schmidt passes there)
        c->D.fg_df = (c->fg_df_on && c->precision == BS_PREC_MIXED && c->prm[0].ppe_precond) ? 1 : 0;
        bs::solve_fgmres(c->D, L, maxit, c->prm[0].ppe_precond ? 2 : 8, c->prm[0].ppe_precond, mg_prec_of(c),
                         c->d_nconv, c->h_pinned, c->evsync);
    } else if (c->precision == BS_PREC_MIXED && c->prm[0].mixed_max_outer > 0)
        bs::solve_mixed(c->D, L, maxit, 8, c->d_nconv, c->h_pinned, c->evsync);
    else
        bs::solve_fp64(c->D, L, maxit, c->prm[0].ppe_precond ? 4 : 8, c->prm[0].ppe_precond, mg_prec_of(c),
                       c->d_nconv, c->h_pinned, c->evsync);
    return 0;
}

// host copy of every scene's dynamic state (t, dt, n for the buffer schedule)
int read_dyn(bs_ctx* ctx) {
    ctx->hdyn.resize(ctx->nscene);
    CK(cudaMemcpyAsync(ctx->hdyn.data(), ctx->D.dyn, sizeof(SceneDyn) * ctx->nscene, cudaMemcpyDeviceToHost,
                       ctx->stream));
    CK(cudaStreamSynchronize(ctx->stream));
    return 0;
}

int zone_exchange(bs_ctx* ctx, int s, int z, long n_now) {
    const auto& Z = ctx->zones[s][z];
    const ScenePar& P = ctx->hpar[s];
    if (n_now + Z.n > P.cap) return fail(ctx, BS_E_CAPACITY, "buffer insertion could exceed the scene's row capacity");
    bs::buffer_exchange(ctx->D, launch_of(ctx), s, P, Z.dev);
    ctx->assembled = false;
    return check_launch(ctx);
}

// main.f90:218-234, after the scalar sub-steps and before projection: zone z
// of a scene exchanges when (told + phase) < k period <= (told + dt + phase);
// hdyn holds each scene's t, dt and n from before the step's time advance
int st_buffers(bs_ctx* ctx) {
    if (!ctx->any_zone) return 0;
    for (int s = 0; s < ctx->nscene; ++s) {
        if (ctx->hdyn[s].hold) continue;
        const double told = ctx->hdyn[s].t, tn = told + ctx->hdyn[s].dt;
        long n = ctx->hdyn[s].n;
        for (int z = 0; z < 2; ++z) {
            auto& Z = ctx->zones[s][z];
            if (!Z.set || !(Z.period > 0)) continue;
            const double kp = (double)Z.next_k * Z.period;
            if (((told + Z.phase) < kp) && ((tn + Z.phase) >= kp)) {
                if (int rc = zone_exchange(ctx, s, z, n)) return rc;
                Z.next_k += 1;
                n += Z.n;   // an upper bound of the new count
            }
        }
    }
    return 0;
}

}  // namespace

extern "C" {

void bs_params_default(bs_params* p) {
    std::memset(p, 0, sizeof(*p));
    p->h = 0.013; p->dl = 0.01; p->dt = 1e-4; p->scalar_on = 1;
    p->rho = 1000.0; p->rhomin = 1000.0; p->rel_den = 1.025; p->rhomax = p->rho * p->rel_den;
    p->g = -9.81; p->mu = 0.001; p->tschmidt = 1.0;
    p->por = 0.38; p->lamk = 600.0; p->d50 = 0.00102;
    p->lamfs = 0.80; p->maxdivr = 2.0; p->csh = 0.50; p->maxshift = 0.1; p->sig1 = 0.20;
    p->xlcutoff = -1e300; p->ytcutoff = 1e300;
    p->ppe_tol = 1e-8; p->ppe_maxit = 5000; p->ppe_stop = BS_STOP_RELRES; p->precision = BS_PREC_FP64;
    p->kmax = 48; p->mixed_inner_tol = 1e-3; p->mixed_max_outer = 0;
    p->wc_gamma = 7.0; p->wc_delta = 0.1;
    p->ppe_solver = BS_SOLVER_BICGSTAB; p->ppe_restart = 150;
    p->buf_release_lo = 1e300; p->buf_release_hi = -1e300;   // never
}

int bs_set_device(int32_t device) {
    int n = 0;
    if (cudaGetDeviceCount(&n) != cudaSuccess || device < 0 || device >= n) return BS_E_ARG;
    return cudaSetDevice(device) == cudaSuccess ? BS_OK : BS_E_CUDA;
}

int bs_create(int32_t nscenes, const bs_params* params, const int32_t* capacity, const int32_t* grain_capacity,
              bs_ctx** out) {
    if (nscenes <= 0 || !params || !capacity || !out) return BS_E_ARG;
    if (nscenes > BS_MG_MAXS) return BS_E_CAPACITY;   // multigrid level tables hold BS_MG_MAXS scenes
    bs_ctx* ctx = new bs_ctx();
    ctx->nscene = nscenes;
    {
        int dev = 0;
        cudaGetDevice(&dev);
        cudaDeviceGetAttribute(&ctx->sm_count, cudaDevAttrMultiProcessorCount, dev);
        cudaGetLastError();
    }
    ctx->prm.assign(params, params + nscenes);
    ctx->zones.resize(nscenes);
    ctx->precision = params[0].precision;
    ctx->kmax = 0;
    for (int s = 0; s < nscenes; ++s) {
        if (params[s].precision != ctx->precision) { delete ctx; return BS_E_ARG; }
        if (params[s].cellx < 4 || params[s].celly < 4 || params[s].h <= 0) { delete ctx; return BS_E_ARG; }
        ctx->kmax = std::max(ctx->kmax, (int)params[s].kmax);
    }
    if (ctx->kmax <= 0 || ctx->kmax > 64) { delete ctx; return BS_E_ARG; }
    // layout
    int row = 0, blk = 0, cell = 0, gr = 0, grp = 0;
    std::vector<int> blk_scene, cell_scene;
    ctx->hpar.resize(nscenes);
    for (int s = 0; s < nscenes; ++s) {
        const bs_params& p = params[s];
        ScenePar& P = ctx->hpar[s];
        std::memset(&P, 0, sizeof(P));
        const int cap = ((std::max(capacity[s], 1) + BS_ALIGN - 1) / BS_ALIGN) * BS_ALIGN;
        fill_par(P, p, ctx->kmax);
        P.cell0 = cell;
        P.row0 = row; P.cap = cap;
        P.nblk = cap / BS_THREADS; P.blk0 = blk;
        P.grp0 = grp;
        grp += (P.nblk + 31) / 32;
        ctx->cellx_cap.push_back(p.cellx);
        ctx->celly_cap.push_back(p.celly);
        for (int b = 0; b < P.nblk; ++b) blk_scene.push_back(s);
        for (int q = 0; q < P.ncell; ++q) cell_scene.push_back(s);
        row += cap;
        blk += P.nblk;
        cell += P.ncell;
        ctx->grain0.push_back(gr);
        const int gc = grain_capacity ? std::max(grain_capacity[s], 0) : 0;
        ctx->gcap.push_back(gc);
        gr += gc;
    }
    ctx->nrow_total = row;
    ctx->nblk_total = blk;
    ctx->ngrp_total = grp;
    ctx->ncell_total = cell;
    ctx->ngrain_total = gr;
    Dev& D = ctx->D;
    const size_t R = row, E = (size_t)row * ctx->kmax, C = cell;
    int rc = 0;
#define A(ptr, n) if (!rc) rc = dalloc(ctx, &D.ptr, n)
    A(x, R); A(y, R); A(xs, R); A(ys, R); A(vx, R); A(vy, R); A(vxs, R); A(vys, R); A(p, R);
    A(mass, R); A(rho, R); A(oden, R); A(ovol, R); A(con, R); A(vol, R); A(nu, R);
    A(tid, R); A(flags, R); A(pid, R); A(cell, R);
    A(x2, R); A(y2, R); A(xs2, R); A(ys2, R); A(vx2, R); A(vy2, R); A(vxs2, R); A(vys2, R); A(p2, R);
    A(mass2, R); A(rho2, R); A(oden2, R); A(ovol2, R); A(con2, R); A(vol2, R); A(nu2, R);
    A(tid2, R); A(flags2, R); A(pid2, R); A(cell2, R);
    A(por, R); A(resx, R); A(resy, R); A(nut, R); A(tke, R); A(varts, R); A(gradvx, R); A(vel, R); A(cdiff, R);
    A(c0, R); A(c1, R); A(c2, R); A(c3, R); A(Dp0, R); A(Dp1, R); A(Dp2, R); A(Dp3, R); A(Dt, R);
    A(rho_new, R); A(vol_new, R); A(con_new, R); A(tden, R); A(whyd, R);
    A(qa, R); A(qu, R); A(qw, R); A(qi, R);
    A(ncount, R); A(nidx, E);
    A(adiag, R); A(rhs, R);
    A(sr, R); A(srhat, R); A(sp, R); A(sp2, R); A(sv, R); A(sv2, R); A(ss, R); A(st, R); A(sxd, R);
    A(cell_start, C); A(cell_end, C); A(cell_start2, C); A(cell_end2, C);
    A(bucket, C * BS_NCAT); A(cell_total, C); A(coderank, R);
    A(cell_maxvel, C); A(cell_maxeddy, C); A(scene_max, (size_t)2 * nscenes);
    {
        int mc = 1;
        for (const ScenePar& P : ctx->hpar) mc = std::max(mc, (P.ncell + BS_SCAN_CHUNK - 1) / BS_SCAN_CHUNK);
        D.scan_chunks = mc;
        A(scan_part, (size_t)mc * nscenes);
    }
    A(gx, (size_t)gr); A(gy, (size_t)gr); A(gv, (size_t)gr); A(gcell_start, C); A(gcell_end, C);
    A(gxr, (size_t)gr); A(gyr, (size_t)gr); A(gpos4, (size_t)gr); A(xr, R); A(yr, R);
    if (ctx->precision == BS_PREC_MIXED) {
        A(pos4, R); A(rec0, R); A(rec1, R); A(rec2, R); A(volf2, R); A(cfa, R); A(cfb, R);
    }
    A(part, (size_t)blk * BS_MAXDOT);
    A(err_word, 1);
#undef A
    const size_t pw = (ctx->precision == BS_PREC_MIXED) ? sizeof(float) : sizeof(double);
    if (!rc) {
        double* tmp;
        rc = dalloc(ctx, &tmp, E);
        D.aval = tmp;
    }
    char* bytes[4];
    for (int q = 0; q < 4 && !rc; ++q) rc = dalloc(ctx, &bytes[q], E * pw);
    if (!rc) { D.ndist = bytes[0]; D.nrinv = bytes[1]; D.nkx = bytes[2]; D.nky = bytes[3]; }
    if (ctx->precision == BS_PREC_MIXED && !rc) {
        float* f;
        rc = dalloc(ctx, &f, E);
        D.aval32 = f;
        if (!rc) rc = dalloc(ctx, &D.aval_lo, E);
        if (!rc) rc = dalloc(ctx, &D.zf, R);
        float** fv[] = {&D.fr, &D.fp, &D.fp2, &D.fv, &D.fv2, &D.fs, &D.ft, &D.fd, &D.frhat};
        for (auto q : fv)
            if (!rc) rc = dalloc(ctx, q, R);
    }
    // multigrid levels: level 1 = the half-cell grid of every scene (2 x 2
    // per search cell), level 2 = the cells, then 2x2 coarsening until every
    // scene has at most 256 coarse cells
    if (!rc) {
        MgDev& M = D.mg;
        std::memset(&M, 0, sizeof(M));
        M.omega = 0.9;
        M.cscale = 1.5;
        M.coarse_sweeps = 10;
        M.pre0 = 1;
        M.prec = 1;
        M.wlev = 2;
        M.post0 = 1;
        // each scene reserves the levels of its creation grid (the largest
        // grid the slot takes, bs_set_scene)
        std::vector<std::vector<std::pair<int, int>>> dims(nscenes);
        ctx->mgrange.assign(nscenes, {});
        int L = 1;
        for (int s = 0; s < nscenes; ++s) {
            dims[s] = mg_dims_of(params[s].cellx, params[s].celly);
            for (auto& d : dims[s]) ctx->mgrange[s].push_back(d.first * d.second);
            L = std::max(L, (int)dims[s].size());
        }
        ctx->mgdims = dims;
        const size_t tw = (ctx->precision == BS_PREC_MIXED) ? sizeof(float) : sizeof(double);
        M.nlev = L;
        M.coarse_max = 256;   // a coarsest level holds at most 256 cells (unless BS_MG_MAXL ends it)
        for (int s = 0; s < nscenes; ++s)
            M.coarse_max = std::max(M.coarse_max, dims[s].back().first * dims[s].back().second);
        for (int l = 1; l <= L && !rc; ++l) {
            std::vector<int> off(nscenes, -1), nxv(nscenes, 0), nyv(nscenes, 0), sc;
            int tot = 0;
            for (int s = 0; s < nscenes; ++s) {
                if ((int)dims[s].size() < l) continue;
                off[s] = tot;
                nxv[s] = dims[s][l - 1].first;
                nyv[s] = dims[s][l - 1].second;
                tot += nxv[s] * nyv[s];
                for (int q = 0; q < nxv[s] * nyv[s]; ++q) sc.push_back(s);
            }
            M.n[l] = tot;
            int *doff, *dnx, *dny, *dsc;
            char *A, *dinv, *rr, *zz;
            if (!rc) rc = dalloc(ctx, &doff, nscenes);
            if (!rc) rc = dalloc(ctx, &dnx, nscenes);
            if (!rc) rc = dalloc(ctx, &dny, nscenes);
            if (!rc) rc = dalloc(ctx, &dsc, tot);
            if (!rc) rc = dalloc(ctx, &A, 9 * (size_t)tot * tw);
            if (!rc) rc = dalloc(ctx, &dinv, (size_t)tot * tw);
            if (!rc) rc = dalloc(ctx, &rr, (size_t)tot * tw);
            if (!rc) rc = dalloc(ctx, &zz, (size_t)tot * tw);
            if (rc) break;
            cudaMemcpy(doff, off.data(), sizeof(int) * nscenes, cudaMemcpyHostToDevice);
            cudaMemcpy(dnx, nxv.data(), sizeof(int) * nscenes, cudaMemcpyHostToDevice);
            cudaMemcpy(dny, nyv.data(), sizeof(int) * nscenes, cudaMemcpyHostToDevice);
            if (tot) cudaMemcpy(dsc, sc.data(), sizeof(int) * tot, cudaMemcpyHostToDevice);
            M.off[l] = doff; M.nx[l] = dnx; M.ny[l] = dny; M.scene_of[l] = dsc;
            M.A[l] = A; M.dinv[l] = dinv; M.r[l] = rr; M.z[l] = zz;
        }
        char *d0, *ad, *xi, *uu, *zz;
        if (!rc) rc = dalloc(ctx, &M.sub, R);
        if (!rc) rc = dalloc(ctx, &M.agg1, R);
        if (!rc) mg_tables(ctx);
        if (!rc) rc = dalloc(ctx, &d0, R * tw);
        if (!rc) rc = dalloc(ctx, &ad, R * tw);
        if (!rc) rc = dalloc(ctx, &xi, R * tw);
        if (!rc) rc = dalloc(ctx, &uu, R * tw);
        if (!rc) rc = dalloc(ctx, &zz, R * tw);
        if (!rc) {
            M.dinv0 = d0;
            M.adiagT = ad;
            M.xin = xi;
            M.u = uu;
            M.zz = zz;
        }
    }
    if (!rc && ctx->precision != BS_PREC_MIXED) {   // FP32 matrix copy for an FP32 V-cycle is mixed-only
        D.aval32 = nullptr;
        D.aval_lo = nullptr;
        D.zf = nullptr;
    }
    ScenePar* dpar = nullptr;
    SceneDyn* ddyn = nullptr;
    int *dbs = nullptr, *dcs = nullptr, *dbd = nullptr;
    if (!rc) rc = dalloc(ctx, &dpar, nscenes);
    if (!rc) rc = dalloc(ctx, &ddyn, nscenes);
    if (!rc) rc = dalloc(ctx, &dbs, blk);
    if (!rc) rc = dalloc(ctx, &dcs, cell);
    if (!rc) rc = dalloc(ctx, &dbd, nscenes);
    if (!rc) rc = dalloc(ctx, &ctx->d_nconv, 4);   // [0] inner, [1] outer converged-scene counters
    if (!rc) rc = dalloc(ctx, &D.loop, 1);
    if (rc) {
        int r2 = rc;
        bs_destroy(ctx);
        return r2;
    }
    cudaMemcpy(dpar, ctx->hpar.data(), sizeof(ScenePar) * nscenes, cudaMemcpyHostToDevice);
    cudaMemcpy(dbs, blk_scene.data(), sizeof(int) * blk, cudaMemcpyHostToDevice);
    cudaMemcpy(dcs, cell_scene.data(), sizeof(int) * cell, cudaMemcpyHostToDevice);
    std::vector<SceneDyn> hd(nscenes);
    for (int s = 0; s < nscenes; ++s) {
        std::memset(&hd[s], 0, sizeof(SceneDyn));
        hd[s].dt = params[s].dt;
        hd[s].t = params[s].t0;
        hd[s].dtsol = params[s].dt;
        hd[s].solsteps = 1;
    }
    cudaMemcpy(ddyn, hd.data(), sizeof(SceneDyn) * nscenes, cudaMemcpyHostToDevice);
    D.par = dpar;
    D.dyn = ddyn;
    D.blk_scene = dbs;
    D.cell_scene = dcs;
    D.blk_done = dbd;
    D.ncell_total = cell;
    D.nrow_total = row;
    D.nblk_total = blk;
    D.nscene = nscenes;
    D.kmax = ctx->kmax;
    D.fg_V = D.fg_Z = D.fg_part = D.fg_gpart = D.fg_small = nullptr;
    D.fg_gdone = nullptr;
    D.fg_m = D.fg_small_n = D.fg_ld = 0;
    cudaStreamCreateWithFlags(&ctx->stream, cudaStreamNonBlocking);
    for (auto& q : ctx->side) cudaStreamCreateWithFlags(&q, cudaStreamNonBlocking);
    for (auto& e : ctx->ev) cudaEventCreate(&e);
    cudaEventCreateWithFlags(&ctx->evsync, cudaEventDisableTiming);
    cudaMallocHost(&ctx->h_pinned, sizeof(int) * (nscenes + 4));
    if (ctx->prm[0].ppe_solver == BS_SOLVER_FGMRES) {
        if (int r2 = fg_ensure(ctx)) {
            bs_destroy(ctx);
            return r2;
        }
    }
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) {
        bs_destroy(ctx);
        return BS_E_CUDA;
    }
    *out = ctx;
    return BS_OK;
}

int bs_destroy(bs_ctx* ctx) {
    if (!ctx) return BS_E_ARG;
    if (ctx->stream) cudaStreamSynchronize(ctx->stream);
    if (ctx->cstream) cudaStreamSynchronize(ctx->cstream);
    for (void* q : ctx->allocs) cudaFree(q);
    for (auto& e : ctx->ev)
        if (e) cudaEventDestroy(e);
    if (ctx->evsync) cudaEventDestroy(ctx->evsync);
    if (ctx->h_pinned) cudaFreeHost(ctx->h_pinned);
    if (ctx->h_snapdyn) cudaFreeHost(ctx->h_snapdyn);
    if (ctx->ev_snap) cudaEventDestroy(ctx->ev_snap);
    for (auto& e : ctx->ev_copied)
        if (e) cudaEventDestroy(e);
    if (ctx->cstream) cudaStreamDestroy(ctx->cstream);
    if (ctx->timer.ready)
        for (auto& e : ctx->timer.ev) cudaEventDestroy(e);
    if (ctx->graph.exec) cudaGraphExecDestroy(ctx->graph.exec);
    for (auto& g : ctx->sgraphs)
        if (g.exec) cudaGraphExecDestroy(g.exec);
    for (auto& q : ctx->side)
        if (q) cudaStreamDestroy(q);
    if (ctx->stream) cudaStreamDestroy(ctx->stream);
    delete ctx;
    return BS_OK;
}

const char* bs_last_error(bs_ctx* ctx) { return ctx ? ctx->err.c_str() : "null context"; }

int bs_upload(bs_ctx* ctx, int32_t s, const bs_state* st, const bs_grains* gr) {
    if (!ctx || s < 0 || s >= ctx->nscene || !st) return BS_E_ARG;
    sg_clear(ctx);
    const bs_params& p = ctx->prm[s];
    const ScenePar& P = ctx->hpar[s];
    const int n = st->n;
    if (n > P.cap) return fail(ctx, BS_E_CAPACITY, "scene larger than its capacity");
    // bin: (cell key, walls first, input order) -- boundary.f90:140-190,
    // internal.f90:73-95 -- as a stable counting sort over 2 buckets per cell
    std::vector<int> bucket(n), ord(n), bstart(2 * (size_t)P.ncell + 1, 0);
    {   // each particle's bucket on the host's cores (independent per particle)
        const int T = std::max(1, std::min(16, std::min((int)std::thread::hardware_concurrency(), n / 16384)));
        std::atomic<int> outside{0};
        auto part = [&](int t) {
            const int q0 = (int)((long)n * t / T), q1 = (int)((long)n * (t + 1) / T);
            for (int q = q0; q < q1; ++q) {
                int ci, cj;
                if (!locate(p, st->x[q], st->y[q], &ci, &cj)) {
                    outside = 1;
                    bucket[q] = 0;
                    continue;
                }
                bucket[q] = 2 * ((cj - 1) * p.celly + (ci - 1)) + (st->tid[q] == BS_TID_FLUID ? 1 : 0);
            }
        };
        std::vector<std::thread> pool;
        for (int t = 1; t < T; ++t) pool.emplace_back(part, t);
        part(0);
        for (auto& th : pool) th.join();
        if (outside) return fail(ctx, BS_E_DOMAIN, "particle outside the interior cell grid");
    }
    for (int q = 0; q < n; ++q) bstart[bucket[q] + 1]++;
    for (size_t b = 0; b < 2 * (size_t)P.ncell; ++b) bstart[b + 1] += bstart[b];
    {
        std::vector<int> fill(bstart.begin(), bstart.end() - 1);
        for (int q = 0; q < n; ++q) ord[fill[bucket[q]]++] = q;
    }
    // cell ranges from the bucket starts (cell c = buckets 2c, 2c+1; empty
    // cells: start == end, ranges stay monotone)
    std::vector<int> cstart(P.ncell), cend(P.ncell);
    for (int c = 0; c < P.ncell; ++c) {
        cstart[c] = P.row0 + bstart[2 * (size_t)c];
        cend[c] = P.row0 + bstart[2 * (size_t)c + 2];
    }
    // the arrays in input order into the alternate buffers, the order and
    // buckets beside them, then one gather kernel places every row
    Dev& D = ctx->D;
    const size_t off = P.row0;
    const double* src[] = {st->x, st->y, st->vx, st->vy, st->p, st->mass, st->rho, st->oden, st->ovol, st->con};
    double* stage[] = {D.x2, D.y2, D.vx2, D.vy2, D.p2, D.mass2, D.rho2, D.oden2, D.ovol2, D.con2};
    for (int f = 0; f < 10; ++f)
        CK(cudaMemcpyAsync(stage[f] + off, src[f], sizeof(double) * n, cudaMemcpyHostToDevice, ctx->stream));
    std::vector<int8_t> tid(n);
    for (int q = 0; q < n; ++q) tid[q] = (int8_t)st->tid[q];
    CK(cudaMemcpyAsync(D.tid2 + off, tid.data(), n, cudaMemcpyHostToDevice, ctx->stream));
    if (st->flags) CK(cudaMemcpyAsync(D.flags2 + off, st->flags, n, cudaMemcpyHostToDevice, ctx->stream));
    if (st->pid) CK(cudaMemcpyAsync(D.pid2 + off, st->pid, sizeof(int) * n, cudaMemcpyHostToDevice, ctx->stream));
    CK(cudaMemcpyAsync(D.cell2 + off, bucket.data(), sizeof(int) * n, cudaMemcpyHostToDevice, ctx->stream));
    CK(cudaMemcpyAsync(D.coderank + off, ord.data(), sizeof(int) * n, cudaMemcpyHostToDevice, ctx->stream));
    CK(cudaMemcpyAsync(D.cell_start + P.cell0, cstart.data(), sizeof(int) * P.ncell, cudaMemcpyHostToDevice,
                       ctx->stream));
    CK(cudaMemcpyAsync(D.cell_end + P.cell0, cend.data(), sizeof(int) * P.ncell, cudaMemcpyHostToDevice,
                       ctx->stream));
    bs::upload_gather(D, launch_of(ctx), P.row0, n, P.cell0, st->flags ? 1 : 0, st->pid ? 1 : 0);
    // grains: sorted by cell
    const int ng = gr ? gr->n : 0;
    if (ng > ctx->gcap[s]) return fail(ctx, BS_E_CAPACITY, "more grains than the grain capacity");
    {
        std::vector<std::pair<int, int>> gk;   // (cell, grain) by cell, input order within (counting sort)
        {
            std::vector<int> gc(ng, -1), gstart((size_t)P.ncell + 1, 0);
            for (int q = 0; q < ng; ++q) {
                int ci, cj;
                if (!locate(p, gr->x[q], gr->y[q], &ci, &cj)) continue;
                gc[q] = (cj - 1) * p.celly + (ci - 1);
                gstart[gc[q] + 1]++;
            }
            for (int c = 0; c < P.ncell; ++c) gstart[c + 1] += gstart[c];
            gk.resize(gstart[P.ncell]);
            for (int q = 0; q < ng; ++q)
                if (gc[q] >= 0) gk[gstart[gc[q]]++] = {gc[q], q};
        }
        const int m = (int)gk.size();
        std::vector<double> gx(m), gy(m), gv(m);
        std::vector<float> gxr(m), gyr(m);
        std::vector<float4> gp4(m);
        std::vector<int> gs(P.ncell, 0), ge(P.ncell, 0), cnt(P.ncell, 0);
        for (int q = 0; q < m; ++q) {
            const int k = gk[q].second;
            gx[q] = gr->x[k];
            gy[q] = gr->y[k];
            gv[q] = gr->mass[k] / gr->rho[k];
            const int cj = gk[q].first / p.celly + 1, ci = gk[q].first % p.celly + 1;
            gxr[q] = (float)(gx[q] - xleft_of(p, cj));
            gyr[q] = (float)(gy[q] - ybot_of(p, ci));
            const float xh = (float)gx[q], yh = (float)gy[q];
            gp4[q] = make_float4(xh, (float)(gx[q] - (double)xh), yh, (float)(gy[q] - (double)yh));
            cnt[gk[q].first]++;
        }
        int acc = ctx->grain0[s];
        for (int c = 0; c < P.ncell; ++c) {
            gs[c] = acc;
            acc += cnt[c];
            ge[c] = acc;
        }
        const int g0 = ctx->grain0[s];
        if (m) {
            CK(cudaMemcpy(D.gx + g0, gx.data(), sizeof(double) * m, cudaMemcpyHostToDevice));
            CK(cudaMemcpy(D.gy + g0, gy.data(), sizeof(double) * m, cudaMemcpyHostToDevice));
            CK(cudaMemcpy(D.gv + g0, gv.data(), sizeof(double) * m, cudaMemcpyHostToDevice));
            CK(cudaMemcpy(D.gxr + g0, gxr.data(), sizeof(float) * m, cudaMemcpyHostToDevice));
            CK(cudaMemcpy(D.gyr + g0, gyr.data(), sizeof(float) * m, cudaMemcpyHostToDevice));
            CK(cudaMemcpy(D.gpos4 + g0, gp4.data(), sizeof(float4) * m, cudaMemcpyHostToDevice));
        }
        CK(cudaMemcpy(D.gcell_start + P.cell0, gs.data(), sizeof(int) * P.ncell, cudaMemcpyHostToDevice));
        CK(cudaMemcpy(D.gcell_end + P.cell0, ge.data(), sizeof(int) * P.ncell, cudaMemcpyHostToDevice));
    }
    SceneDyn hd;
    std::memset(&hd, 0, sizeof(hd));
    hd.n = n;
    hd.t = p.t0;
    hd.dt = p.dt;
    hd.dtsol = p.dt;
    hd.solsteps = 1;
    CK(cudaMemcpy(D.dyn + s, &hd, sizeof(hd), cudaMemcpyHostToDevice));
    bs::derive_fields(D, launch_of(ctx));
    CK(cudaStreamSynchronize(ctx->stream));
    ctx->assembled = false;
    return check_launch(ctx);
}

int bs_download_async(bs_ctx* ctx, int32_t s, bs_state* o) {
    if (!ctx || s < 0 || s >= ctx->nscene || !o) return BS_E_ARG;
    if (o->cell || o->coff) return fail(ctx, BS_E_ARG, "cell and coff are not read back asynchronously");
    const ScenePar& P = ctx->hpar[s];
    if (o->n < P.cap) return fail(ctx, BS_E_CAPACITY, "asynchronous read-back buffers hold fewer rows than the scene's capacity");
    Dev& D = ctx->D;
    const size_t R = ctx->nrow_total;
    double* outs[BS_SNAP_MAXF] = {o->x, o->y, o->vx, o->vy, o->p, o->mass, o->rho, o->oden, o->ovol, o->con,
                                  o->xs, o->ys, o->vxs, o->vys, o->porosity, o->resx, o->resy, o->nut, o->tke,
                                  o->varts, o->gradvx, o->vel, o->cdiff};
    const double* srcs[BS_SNAP_MAXF] = {D.x, D.y, D.vx, D.vy, D.p, D.mass, D.rho, D.oden, D.ovol, D.con,
                                        D.xs, D.ys, D.vxs, D.vys, D.por, D.resx, D.resy, D.nut, D.tke,
                                        D.varts, D.gradvx, D.vel, D.cdiff};
    if (!ctx->snap) {   // first use: snapshot buffer, copy stream, events, pinned dynamic state
        const size_t bytes = R * (BS_SNAP_MAXF * sizeof(double) + 2 * sizeof(int) + 1) +
                             sizeof(SceneDyn) * (size_t)ctx->nscene + 256;
        if (int rc = dalloc(ctx, &ctx->snap, bytes)) return rc;
        CK(cudaStreamCreateWithFlags(&ctx->cstream, cudaStreamNonBlocking));
        CK(cudaEventCreateWithFlags(&ctx->ev_snap, cudaEventDisableTiming));
        ctx->ev_copied.assign(ctx->nscene, nullptr);
        for (auto& e : ctx->ev_copied) CK(cudaEventCreateWithFlags(&e, cudaEventDisableTiming));
        CK(cudaMallocHost(&ctx->h_snapdyn, sizeof(SceneDyn) * (size_t)ctx->nscene));
    }
    char* base = ctx->snap;
    double* fsnap = (double*)base;                                  // field f: fsnap + f R
    int* tsnap = (int*)(base + R * BS_SNAP_MAXF * sizeof(double));  // tid, then pid
    uint8_t* flsnap = (uint8_t*)(tsnap + 2 * R);
    SceneDyn* dsnap = (SceneDyn*)(((uintptr_t)(flsnap + R) + 255) & ~(uintptr_t)255);
    // the scene's previous read-back must have left its rows of the snapshot
    CK(cudaStreamWaitEvent(ctx->stream, ctx->ev_copied[s], 0));
    bs::SnapArgs a{};
    int fidx[BS_SNAP_MAXF];
    for (int f = 0; f < BS_SNAP_MAXF; ++f)
        if (outs[f]) {
            fidx[a.nf] = f;
            a.src[a.nf] = srcs[f];
            a.dst[a.nf] = fsnap + (size_t)f * R;
            a.nf++;
        }
    a.row0 = P.row0;
    a.n = P.cap;
    if (o->tid) { a.tid = D.tid; a.tid_dst = tsnap; }
    if (o->pid) { a.pid = D.pid; a.pid_dst = tsnap + R; }
    if (o->flags) { a.flags = D.flags; a.flags_dst = flsnap; }
    bs::snapshot(launch_of(ctx), a);
    CK(cudaMemcpyAsync(dsnap + s, D.dyn + s, sizeof(SceneDyn), cudaMemcpyDeviceToDevice, ctx->stream));
    CK(cudaEventRecord(ctx->ev_snap, ctx->stream));
    // the copy to the host on the copy stream, behind the snapshot
    CK(cudaStreamWaitEvent(ctx->cstream, ctx->ev_snap, 0));
    const size_t off = P.row0, n = (size_t)P.cap;
    for (int k = 0; k < a.nf; ++k)
        CK(cudaMemcpyAsync(outs[fidx[k]], fsnap + (size_t)fidx[k] * R + off, sizeof(double) * n,
                           cudaMemcpyDeviceToHost, ctx->cstream));
    if (o->tid) CK(cudaMemcpyAsync(o->tid, tsnap + off, sizeof(int) * n, cudaMemcpyDeviceToHost, ctx->cstream));
    if (o->pid) CK(cudaMemcpyAsync(o->pid, tsnap + R + off, sizeof(int) * n, cudaMemcpyDeviceToHost, ctx->cstream));
    if (o->flags) CK(cudaMemcpyAsync(o->flags, flsnap + off, n, cudaMemcpyDeviceToHost, ctx->cstream));
    CK(cudaMemcpyAsync(ctx->h_snapdyn + s, dsnap + s, sizeof(SceneDyn), cudaMemcpyDeviceToHost, ctx->cstream));
    CK(cudaEventRecord(ctx->ev_copied[s], ctx->cstream));
    return check_launch(ctx);
}

int bs_download_wait(bs_ctx* ctx, int32_t s, bs_state* o) {
    if (!ctx || s < 0 || s >= ctx->nscene || !o) return BS_E_ARG;
    if (ctx->ev_copied.empty()) return fail(ctx, BS_E_ARG, "no asynchronous read-back was started");
    CK(cudaEventSynchronize(ctx->ev_copied[s]));
    o->n = ctx->h_snapdyn[s].n;
    return 0;
}

int bs_host_alloc(size_t bytes, void** p) {
    if (!p) return BS_E_ARG;
    *p = nullptr;
    if (cudaMallocHost(p, bytes ? bytes : 1) != cudaSuccess) {
        cudaGetLastError();
        *p = nullptr;
        return BS_E_NOMEM;
    }
    return 0;
}
int bs_host_free(void* p) {
    if (p && cudaFreeHost(p) != cudaSuccess) {
        cudaGetLastError();
        return BS_E_CUDA;
    }
    return 0;
}

int bs_download(bs_ctx* ctx, int32_t s, bs_state* o) {
    if (!ctx || s < 0 || s >= ctx->nscene || !o) return BS_E_ARG;
    CK(cudaStreamSynchronize(ctx->stream));
    SceneDyn hd;
    CK(cudaMemcpy(&hd, ctx->D.dyn + s, sizeof(hd), cudaMemcpyDeviceToHost));
    const int n = hd.n;
    if (o->n < n) return fail(ctx, BS_E_CAPACITY, "download buffer too small");
    o->n = n;
    const size_t off = ctx->hpar[s].row0;
    Dev& D = ctx->D;
    // stream-ordered copies and one synchronisation: into pinned buffers
    // (bs_host_alloc) they overlap and run at the host link's rate
    auto get = [&](double* dst, const double* src) -> int {
        if (!dst) return 0;
        cudaError_t e = cudaMemcpyAsync(dst, src + off, sizeof(double) * n, cudaMemcpyDeviceToHost, ctx->stream);
        return e == cudaSuccess ? 0 : BS_E_CUDA;
    };
    int rc = 0;
    rc |= get(o->x, D.x); rc |= get(o->y, D.y); rc |= get(o->vx, D.vx); rc |= get(o->vy, D.vy);
    rc |= get(o->p, D.p); rc |= get(o->mass, D.mass); rc |= get(o->rho, D.rho); rc |= get(o->oden, D.oden);
    rc |= get(o->ovol, D.ovol); rc |= get(o->con, D.con); rc |= get(o->xs, D.xs); rc |= get(o->ys, D.ys);
    rc |= get(o->vxs, D.vxs); rc |= get(o->vys, D.vys); rc |= get(o->porosity, D.por); rc |= get(o->resx, D.resx);
    rc |= get(o->resy, D.resy); rc |= get(o->nut, D.nut); rc |= get(o->tke, D.tke); rc |= get(o->varts, D.varts);
    rc |= get(o->gradvx, D.gradvx); rc |= get(o->vel, D.vel); rc |= get(o->cdiff, D.cdiff);
    if (rc) return fail(ctx, BS_E_CUDA, "download copy failed");
    if (o->flags) CK(cudaMemcpyAsync(o->flags, D.flags + off, n, cudaMemcpyDeviceToHost, ctx->stream));
    if (o->pid) CK(cudaMemcpyAsync(o->pid, D.pid + off, sizeof(int) * n, cudaMemcpyDeviceToHost, ctx->stream));
    CK(cudaStreamSynchronize(ctx->stream));
    if (o->tid) {
        std::vector<int8_t> t(n);
        CK(cudaMemcpy(t.data(), D.tid + off, n, cudaMemcpyDeviceToHost));
        for (int q = 0; q < n; ++q) o->tid[q] = t[q];
    }
    if (o->cell) {
        CK(cudaMemcpy(o->cell, D.cell + off, sizeof(int) * n, cudaMemcpyDeviceToHost));
        for (int q = 0; q < n; ++q) o->cell[q] -= ctx->hpar[s].cell0;
    }
    if (o->coff) {
        std::vector<double> c[4];
        double* src[4] = {D.c0, D.c1, D.c2, D.c3};
        for (int k = 0; k < 4; ++k) {
            c[k].resize(n);
            CK(cudaMemcpy(c[k].data(), src[k] + off, sizeof(double) * n, cudaMemcpyDeviceToHost));
        }
        for (int q = 0; q < n; ++q)
            for (int k = 0; k < 4; ++k) o->coff[4 * q + k] = c[k][q];
    }
    return 0;
}

int bs_scene_info_get(bs_ctx* ctx, int32_t s, bs_scene_info* o) {
    if (!ctx || s < 0 || s >= ctx->nscene || !o) return BS_E_ARG;
    CK(cudaStreamSynchronize(ctx->stream));
    SceneDyn hd;
    CK(cudaMemcpy(&hd, ctx->D.dyn + s, sizeof(hd), cudaMemcpyDeviceToHost));
    std::memset(o, 0, sizeof(*o));
    o->n = hd.n;
    o->solsteps = hd.solsteps;
    o->ppe_iters = hd.iters;
    o->ppe_outer = hd.outer < 0 ? -hd.outer - 1 : hd.outer;
    o->dt = hd.dt;
    o->dtsol = hd.dtsol;
    o->t = hd.t;
    o->umax = hd.umax;
    o->numax = hd.numax;
    o->ppe_relres = hd.relres;
    o->err_bits = hd.err;
    return 0;
}

int bs_clear_errors(bs_ctx* ctx) {
    if (!ctx) return BS_E_ARG;
    CK(cudaStreamSynchronize(ctx->stream));
    std::vector<SceneDyn> hd(ctx->nscene);
    CK(cudaMemcpy(hd.data(), ctx->D.dyn, sizeof(SceneDyn) * ctx->nscene, cudaMemcpyDeviceToHost));
    for (auto& d : hd) d.err = 0;
    CK(cudaMemcpy(ctx->D.dyn, hd.data(), sizeof(SceneDyn) * ctx->nscene, cudaMemcpyHostToDevice));
    CK(cudaMemset(ctx->D.err_word, 0, sizeof(unsigned)));
    return 0;
}

int bs_sync(bs_ctx* ctx) {
    if (!ctx) return BS_E_ARG;
    CK(cudaStreamSynchronize(ctx->stream));
    return check_launch(ctx);
}

int bs_get_neighbours(bs_ctx* ctx, int32_t s, int32_t* counts, int32_t* idx, double* dist, double* kx, double* ky) {
    if (!ctx || s < 0 || s >= ctx->nscene) return BS_E_ARG;
    CK(cudaStreamSynchronize(ctx->stream));
    SceneDyn hd;
    CK(cudaMemcpy(&hd, ctx->D.dyn + s, sizeof(hd), cudaMemcpyDeviceToHost));
    const ScenePar& P = ctx->hpar[s];
    const int n = hd.n, K = ctx->kmax;
    const size_t e0 = (size_t)P.row0 * K, ne = (size_t)P.cap * K;
    std::vector<int> cnt(n), id(ne);
    CK(cudaMemcpy(cnt.data(), ctx->D.ncount + P.row0, sizeof(int) * n, cudaMemcpyDeviceToHost));
    CK(cudaMemcpy(id.data(), ctx->D.nidx + e0, sizeof(int) * ne, cudaMemcpyDeviceToHost));
    const bool mixed = ctx->precision == BS_PREC_MIXED;
    std::vector<double> vals[3];
    void* srcs[3] = {ctx->D.ndist, ctx->D.nkx, ctx->D.nky};
    double* outs[3] = {dist, kx, ky};
    for (int q = 0; q < 3; ++q) {
        if (!outs[q]) continue;
        vals[q].resize(ne);
        if (mixed) {
            std::vector<float> f(ne);
            CK(cudaMemcpy(f.data(), (float*)srcs[q] + e0, sizeof(float) * ne, cudaMemcpyDeviceToHost));
            for (size_t e = 0; e < ne; ++e) vals[q][e] = f[e];
        } else {
            CK(cudaMemcpy(vals[q].data(), (double*)srcs[q] + e0, sizeof(double) * ne, cudaMemcpyDeviceToHost));
        }
    }
    for (int r = 0; r < n; ++r) {
        if (counts) counts[r] = cnt[r];
        for (int k = 0; k < cnt[r]; ++k) {
            const size_t e = ((size_t)(r >> 5) * K + k) * 32 + (r & 31);
            const size_t o = (size_t)r * K + k;
            if (idx) idx[o] = id[e] - P.row0;
            for (int q = 0; q < 3; ++q)
                if (outs[q]) outs[q][o] = vals[q][e];
        }
    }
    return 0;
}

int bs_get_matrix(bs_ctx* ctx, int32_t s, double* diag, double* off, double* rhs) {
    if (!ctx || s < 0 || s >= ctx->nscene) return BS_E_ARG;
    if (!ctx->assembled) return fail(ctx, BS_E_STATE, "matrix not assembled");
    CK(cudaStreamSynchronize(ctx->stream));
    SceneDyn hd;
    CK(cudaMemcpy(&hd, ctx->D.dyn + s, sizeof(hd), cudaMemcpyDeviceToHost));
    const ScenePar& P = ctx->hpar[s];
    const int n = hd.n, K = ctx->kmax;
    if (diag) CK(cudaMemcpy(diag, ctx->D.adiag + P.row0, sizeof(double) * n, cudaMemcpyDeviceToHost));
    if (rhs) CK(cudaMemcpy(rhs, ctx->D.rhs + P.row0, sizeof(double) * n, cudaMemcpyDeviceToHost));
    if (off) {
        const size_t e0 = (size_t)P.row0 * K, ne = (size_t)P.cap * K;
        std::vector<double> v(ne);
        std::vector<int> cnt(n);
        CK(cudaMemcpy(v.data(), (double*)ctx->D.aval + e0, sizeof(double) * ne, cudaMemcpyDeviceToHost));
        CK(cudaMemcpy(cnt.data(), ctx->D.ncount + P.row0, sizeof(int) * n, cudaMemcpyDeviceToHost));
        for (int r = 0; r < n; ++r)
            for (int k = 0; k < cnt[r]; ++k) off[(size_t)r * K + k] = v[((size_t)(r >> 5) * K + k) * 32 + (r & 31)];
    }
    return 0;
}

// Tunables of the solver (set by the autotuner, autotune.py).
int bs_set_option(bs_ctx* ctx, const char* name, double value) {
    if (!ctx || !name) return BS_E_ARG;
    CK(cudaStreamSynchronize(ctx->stream));
    MgDev& M = ctx->D.mg;
    const std::string k(name);
    if (k == "mg_omega" && value > 0 && value < 2) M.omega = value;
    else if (k == "mg_cscale" && value > 0 && value < 4) M.cscale = value;
    else if (k == "mg_pre0") M.pre0 = value != 0;
    else if (k == "mg_prec") M.prec = value != 0;
    else if (k == "mg_coarse_sweeps" && value >= 1 && value <= 1000) M.coarse_sweeps = (int)value;
    else if (k == "mg_wlev" && value >= 0 && value <= BS_MG_MAXL) M.wlev = (int)value;
    else if (k == "mg_post0" && (value == 1 || value == 2)) M.post0 = (int)value;
    else if (k == "ppe_precond") for (auto& p : ctx->prm) p.ppe_precond = (int32_t)value;
    else if (k == "mg_sub" && (value == 0 || value == 1)) ctx->mgsub_on = (int)value;
    else if (k == "fg_df" && (value == 0 || value == 1)) ctx->fg_df_on = (int)value;
    else if (k == "mg_tail" && (value == 0 || value == 1)) ctx->mgtail_on = (int)value;
    else if (k == "mg_fp32" && (value == 0 || value == 1)) {
        if (value == 1 && ctx->precision != BS_PREC_MIXED && !ctx->D.aval32) {   // the FP32 matrix copy
            const size_t E = (size_t)ctx->nrow_total * ctx->kmax;
            if (int rc = dalloc(ctx, &ctx->D.aval32, E)) return rc;
            if (int rc = dalloc(ctx, &ctx->D.aval_lo, E)) return rc;
        }
        ctx->mg_fp32 = (int)value;
    }
    else if (k == "ppe_solver" && (value == BS_SOLVER_BICGSTAB || value == BS_SOLVER_FGMRES))
        for (auto& p : ctx->prm) p.ppe_solver = (int32_t)value;
    else if (k == "ppe_restart" && value >= 1 && value <= BS_FG_MAXM)
        for (auto& p : ctx->prm) p.ppe_restart = (int32_t)value;
    else if (k == "mg_exact" && (value == 0 || value == 1)) {
        if (value == 1 && !M.ainv) {
            const size_t per = (size_t)BS_MG_EXACT_MAX * BS_MG_EXACT_MAX * ctx->nscene;
            int rc = bs::mg_exact_prepare();
            if (rc) return fail(ctx, rc, "exact coarse solve: shared memory attribute");
            char* a = nullptr;
            rc = dalloc(ctx, &a, per * (ctx->precision == BS_PREC_MIXED ? sizeof(float) : sizeof(double)));
            if (!rc) rc = dalloc(ctx, &M.xinv, per);
            if (rc) return rc;
            M.ainv = a;
        }
        M.exact = (int)value;
        if (!ctx->mglev.empty()) mg_tables(ctx);
    }
    else if ((k == "sweep_tpb" || k == "mg0_tpb") && (value == 64 || value == 128 || value == 256))
        (k == "sweep_tpb" ? ctx->sweep_tpb : ctx->mg0_tpb) = (int)value;
    else if (k == "step_graph" && (value == 0 || value == 1)) {
        ctx->step_graph_on = (int)value;
        ctx->step_graph_broken = false;
    } else return fail(ctx, BS_E_ARG, "unknown option or value out of range: " + k);
    sg_clear(ctx);
    if (ctx->prm[0].ppe_solver == BS_SOLVER_FGMRES)
        if (int rc = fg_ensure(ctx)) return rc;
    mg_sub_choose(ctx);   // the W depth changes the visits' op lists
    mg_tail_choose(ctx);
    ctx->graph.valid = false;   // the captured iteration holds the old values
    return 0;
}

int bs_get_option(bs_ctx* ctx, const char* name, double* value) {
    if (!ctx || !name || !value) return BS_E_ARG;
    const MgDev& M = ctx->D.mg;
    const std::string k(name);
    if (k == "mg_omega") *value = M.omega;
    else if (k == "mg_cscale") *value = M.cscale;
    else if (k == "mg_pre0") *value = M.pre0;
    else if (k == "mg_prec") *value = M.prec;
    else if (k == "mg_coarse_sweeps") *value = M.coarse_sweeps;
    else if (k == "mg_wlev") *value = M.wlev;
    else if (k == "mg_post0") *value = M.post0;
    else if (k == "mg_levels") *value = M.nlev;
    else if (k == "ppe_precond") *value = ctx->prm[0].ppe_precond;
    else if (k == "ppe_solver") *value = ctx->prm[0].ppe_solver;
    else if (k == "mg_sub") *value = ctx->mgsub_on;
    else if (k == "fg_df") *value = ctx->fg_df_on;
    else if (k == "mg_tail") *value = ctx->mgtail_on;
    else if (k == "mg_tail_level") *value = ctx->mgtail_level;
    else if (k == "mg_fp32") *value = ctx->mg_fp32;
    else if (k == "mg_sub_level") *value = ctx->mgsub_level;
    else if (k == "ppe_restart") *value = ctx->prm[0].ppe_restart;
    else if (k == "mg_exact") *value = M.exact;
    else if (k == "sweep_tpb") *value = ctx->sweep_tpb;
    else if (k == "mg0_tpb") *value = ctx->mg0_tpb;
    else if (k == "step_graph") *value = ctx->step_graph_on && !ctx->step_graph_broken;
    else if (k == "step_graph_steps") *value = (double)ctx->graph_steps;
    else if (k == "step_graph_cached") *value = (double)ctx->sgraphs.size();
    else return BS_E_ARG;
    return 0;
}

int bs_set_rhs(bs_ctx* ctx, int32_t s, const double* b) {
    if (!ctx || s < 0 || s >= ctx->nscene || !b) return BS_E_ARG;
    if (!ctx->assembled) return fail(ctx, BS_E_STATE, "matrix not assembled");
    CK(cudaStreamSynchronize(ctx->stream));
    SceneDyn hd;
    CK(cudaMemcpy(&hd, ctx->D.dyn + s, sizeof(hd), cudaMemcpyDeviceToHost));
    CK(cudaMemcpy(ctx->D.rhs + ctx->hpar[s].row0, b, sizeof(double) * hd.n, cudaMemcpyHostToDevice));
    return 0;
}

// Buffer zone of a scene (remove_bufferN / insert_bufferN, internal.f90:447-586):
// entry-cell bits per cell, the template grouped by destination cell (template
// order within a cell; particles outside the entry cells dropped, as the
// reference only visits entry cells), uploaded once.
int bs_set_inflow(bs_ctx* ctx, int32_t s, int32_t zone, const bs_inflow* z) {
    if (!ctx || s < 0 || s >= ctx->nscene || zone < 0 || zone > 1 || !z || z->n < 0 || z->ncells < 0)
        return BS_E_ARG;
    sg_clear(ctx);
    const bool clear = (z->n == 0 && z->ncells == 0);
    if (!clear && ((z->n && (!z->x || !z->y || !z->vx || !z->vy || !z->p)) || (z->ncells && (!z->cell_i || !z->cell_j)) ||
                   (z->remove_side != 1 && z->remove_side != -1) || !(z->rho > 0)))
        return fail(ctx, BS_E_ARG, "bad buffer zone");
    CK(cudaStreamSynchronize(ctx->stream));
    Dev& D = ctx->D;
    if (!D.czone) {
        int rc = dalloc(ctx, &D.czone, ctx->ncell_total);
        for (int q = 0; q < 2 && !rc; ++q) {
            rc = dalloc(ctx, &D.zstart[q], ctx->ncell_total);
            if (!rc) rc = dalloc(ctx, &D.zcount[q], ctx->ncell_total);
        }
        if (rc) return rc;
    }
    const ScenePar& P = ctx->hpar[s];
    const bs_params& p = ctx->prm[s];
    const uint8_t bit = (uint8_t)(1u << zone);
    std::vector<uint8_t> cz(P.ncell);
    CK(cudaMemcpy(cz.data(), D.czone + P.cell0, P.ncell, cudaMemcpyDeviceToHost));
    for (auto& b : cz) b &= (uint8_t)~bit;
    std::vector<int> zst(P.ncell, 0), zct(P.ncell, 0);
    std::vector<double> tf[5];
    std::vector<int> tpid;
    if (!clear) {
        for (int q = 0; q < z->ncells; ++q) {
            const int i = z->cell_i[q], j = z->cell_j[q];
            if (i < 2 || i > p.celly - 1 || j < 2 || j > p.cellx - 1)
                return fail(ctx, BS_E_ARG, "entry cell outside the interior grid");
            const int lc = (j - 1) * p.celly + (i - 1);
            if (cz[lc] & bit) return fail(ctx, BS_E_ARG, "entry cell listed twice");
            cz[lc] |= bit;
        }
        std::vector<std::pair<int, int>> order;   // (cell, template index)
        for (int q = 0; q < z->n; ++q) {
            int ci, cj;
            if (!locate(p, z->x[q], z->y[q], &ci, &cj)) continue;
            const int lc = (cj - 1) * p.celly + (ci - 1);
            if (cz[lc] & bit) order.push_back({lc, q});
        }
        std::stable_sort(order.begin(), order.end(),
                         [](const std::pair<int, int>& a, const std::pair<int, int>& b) { return a.first < b.first; });
        for (size_t k = 0; k < order.size(); ++k) {
            const int lc = order[k].first, q = order[k].second;
            if (zct[lc] == 0) zst[lc] = (int)k;
            zct[lc]++;
            tf[0].push_back(z->x[q]);
            tf[1].push_back(z->y[q]);
            tf[2].push_back(z->vx[q]);
            tf[3].push_back(z->vy[q]);
            tf[4].push_back(z->p[q]);
            tpid.push_back(z->pid ? z->pid[q] : 0);
        }
    }
    CK(cudaMemcpy(D.czone + P.cell0, cz.data(), P.ncell, cudaMemcpyHostToDevice));
    CK(cudaMemcpy(D.zstart[zone] + P.cell0, zst.data(), sizeof(int) * P.ncell, cudaMemcpyHostToDevice));
    CK(cudaMemcpy(D.zcount[zone] + P.cell0, zct.data(), sizeof(int) * P.ncell, cudaMemcpyHostToDevice));
    auto& Z = ctx->zones[s][zone];
    dfree(ctx, Z.mem);
    dfree(ctx, Z.pmem);
    Z = bs_ctx::Zone();
    if (!clear) {
        const size_t m = tf[0].size();
        int rc = dalloc(ctx, &Z.mem, 5 * m);
        if (!rc) rc = dalloc(ctx, &Z.pmem, m);
        if (rc) return rc;
        for (int f = 0; f < 5; ++f)
            if (m) CK(cudaMemcpy(Z.mem + f * m, tf[f].data(), sizeof(double) * m, cudaMemcpyHostToDevice));
        if (m) CK(cudaMemcpy(Z.pmem, tpid.data(), sizeof(int) * m, cudaMemcpyHostToDevice));
        bs::ZoneDev& G = Z.dev;
        G.x = Z.mem;
        G.y = Z.mem + m;
        G.vx = Z.mem + 2 * m;
        G.vy = Z.mem + 3 * m;
        G.p = Z.mem + 4 * m;
        G.pid = Z.pmem;
        G.mass = z->mass;
        G.rho = z->rho;
        G.ovol = z->ovol;
        G.con = z->con;
        G.remove_x = z->remove_x;
        G.remove_side = z->remove_side;
        G.zone = zone;
        Z.period = z->period;
        Z.phase = z->phase;
        Z.next_k = 1;
        Z.n = (int)m;
        Z.set = true;
    }
    ctx->any_zone = false;
    for (auto& a : ctx->zones)
        for (auto& b : a) ctx->any_zone |= b.set;
    return 0;
}

int bs_buffer_exchange(bs_ctx* ctx, int32_t s, int32_t zone) {
    if (!ctx || s < 0 || s >= ctx->nscene || zone < 0 || zone > 1) return BS_E_ARG;
    if (!ctx->zones[s][zone].set) return fail(ctx, BS_E_STATE, "buffer zone not set");
    if (int rc = read_dyn(ctx)) return rc;
    if (int rc = zone_exchange(ctx, s, zone, ctx->hdyn[s].n)) return rc;
    return bs_sync(ctx);
}

// Re-use scene slot s for another scene: new parameters (its cell grid no
// larger than the one the slot was created with), particles and grains.
int bs_set_scene(bs_ctx* ctx, int32_t s, const bs_params* p, const bs_state* st, const bs_grains* gr) {
    if (!ctx || s < 0 || s >= ctx->nscene || !p || !st) return BS_E_ARG;
    if (p->precision != ctx->precision || p->kmax > ctx->kmax || p->h <= 0 || p->cellx < 4 || p->celly < 4)
        return fail(ctx, BS_E_ARG, "scene parameters do not fit this context");
    if (p->cellx > ctx->cellx_cap[s] || p->celly > ctx->celly_cap[s])
        return fail(ctx, BS_E_CAPACITY, "cell grid larger than the slot's");
    if (st->n > ctx->hpar[s].cap) return fail(ctx, BS_E_CAPACITY, "scene larger than its capacity");
    if (gr && gr->n > ctx->gcap[s]) return fail(ctx, BS_E_CAPACITY, "more grains than the grain capacity");
    CK(cudaStreamSynchronize(ctx->stream));
    Dev& D = ctx->D;
    ScenePar& P = ctx->hpar[s];
    // empty every reserved cell of the slot (cells beyond the new grid stay empty)
    const size_t nc = (size_t)ctx->cellx_cap[s] * ctx->celly_cap[s];
    int* zc[] = {D.cell_start, D.cell_end, D.cell_start2, D.cell_end2, D.gcell_start, D.gcell_end, D.cell_total};
    for (int* a : zc) CK(cudaMemset(a + P.cell0, 0, sizeof(int) * nc));
    CK(cudaMemset(D.cell_maxvel + P.cell0, 0, sizeof(double) * nc));
    CK(cudaMemset(D.cell_maxeddy + P.cell0, 0, sizeof(double) * nc));
    for (int z = 0; z < 2; ++z)   // the slot's buffer zones belong to the old scene
        if (ctx->zones[s][z].set) {
            bs_inflow none;
            std::memset(&none, 0, sizeof(none));
            if (int rc = bs_set_inflow(ctx, s, z, &none)) return rc;
        }
    ctx->prm[s] = *p;
    fill_par(P, *p, ctx->kmax);
    ctx->mgdims[s] = mg_dims_of(p->cellx, p->celly);
    mg_tables(ctx);
    CK(cudaMemcpy((void*)(D.par + s), &P, sizeof(ScenePar), cudaMemcpyHostToDevice));
    ctx->graph.valid = false;   // the level tables are baked into the captured chunk
    ctx->assembled = false;
    return bs_upload(ctx, s, st, gr);
}

// ------------------------------------------------------------------ output
namespace {
// Fortran Fw.d / ESw.d edit descriptors as gfortran prints them: right
// justified in w columns, asterisks when the value does not fit
void fortran_f(std::string& out, double v, int w, int d) {
    char b[64];
    std::snprintf(b, sizeof b, "%*.*f", w, d, v);
    out += (int)std::strlen(b) > w ? std::string(w, '*') : std::string(b);
}
void fortran_es(std::string& out, double v, int w, int d) {
    char b[64];
    std::snprintf(b, sizeof b, "%*.*E", w, d, v);
    out += (int)std::strlen(b) > w ? std::string(w, '*') : std::string(b);
}
}  // namespace

int bs_write_combined(bs_ctx* ctx, int32_t s, const char* fluid_path, const char* buffer_path) {
    if (!ctx || s < 0 || s >= ctx->nscene || !fluid_path) return BS_E_ARG;
    SceneDyn hd;
    CK(cudaStreamSynchronize(ctx->stream));
    CK(cudaMemcpy(&hd, ctx->D.dyn + s, sizeof(hd), cudaMemcpyDeviceToHost));
    const int n = hd.n, off = ctx->hpar[s].row0;
    const Dev& D = ctx->D;
    std::vector<double> x(n), y(n), p(n), vx(n), vy(n), con(n);
    std::vector<int8_t> tid(n);
    std::vector<uint8_t> fl(n);
    double* dst[] = {x.data(), y.data(), p.data(), vx.data(), vy.data(), con.data()};
    const double* src[] = {D.x, D.y, D.p, D.vx, D.vy, D.con};
    for (int f = 0; f < 6; ++f)
        if (n) CK(cudaMemcpy(dst[f], src[f] + off, sizeof(double) * n, cudaMemcpyDeviceToHost));
    if (n) CK(cudaMemcpy(tid.data(), D.tid + off, n, cudaMemcpyDeviceToHost));
    if (n) CK(cudaMemcpy(fl.data(), D.flags + off, n, cudaMemcpyDeviceToHost));
    FILE* ff = std::fopen(fluid_path, "w");
    if (!ff) return fail(ctx, BS_E_ARG, std::string("cannot write ") + fluid_path);
    FILE* fb = buffer_path ? std::fopen(buffer_path, "w") : nullptr;
    std::string line;
    // rows are in the reference's order: columns of cells, rows of cells,
    // slots (output.f90:199-216)
    for (int q = 0; q < n; ++q) {
        if (tid[q] != BS_TID_FLUID) continue;
        const bool buf = (fl[q] & BS_FLAG_BUFFER) != 0;
        FILE* f = buf ? fb : ff;
        if (!f) continue;
        line.clear();
        fortran_f(line, x[q], 10, 3); line += ' ';
        fortran_f(line, y[q], 10, 3); line += ' ';
        fortran_f(line, p[q], 10, 3); line += ' ';
        fortran_es(line, vx[q], 10, 3); line += ' ';
        fortran_es(line, vy[q], 10, 3); line += ' ';
        fortran_f(line, con[q] + 0.50, 10, 5);
        line += '\n';
        std::fputs(line.c_str(), f);
    }
    std::fclose(ff);
    if (fb) std::fclose(fb);
    return 0;
}

// ------------------------------------------------------------------ stages
static int prime_impl(bs_ctx* ctx, int rule) {
    if (!ctx) return BS_E_ARG;
    bs::Launch L = launch_of(ctx);
    st_search(ctx, 1, 1);
    bs::eddy(ctx->D, L, ctx->precision, 1, 0, 0);
    bs::velmag(ctx->D, L);
    bs::cell_max_timestep(ctx->D, L, 1, rule);
    bs::disp(ctx->D, L);
    ctx->disp_ready = true;
    int rc = check_launch(ctx);
    if (rc) return rc;
    return read_solsteps(ctx);
}

int bs_prime(bs_ctx* ctx) { return prime_impl(ctx, 1); }

// The reference's set-up (main.f90:23-37) leaves dt at its initial value and
// umax at 0 for the first step: prime without the time-step rule.
int bs_prime_setup(bs_ctx* ctx) { return prime_impl(ctx, 0); }

// Prime one scene only: the others are held (their rows, cells and
// timestep untouched), so scenes already stepping carry on exactly as if no
// other scene had joined.
int bs_prime_scene(bs_ctx* ctx, int32_t s) {
    if (!ctx || s < 0 || s >= ctx->nscene) return BS_E_ARG;
    CK(cudaStreamSynchronize(ctx->stream));
    const size_t off = offsetof(SceneDyn, hold);
    for (int k = 0; k < ctx->nscene; ++k) {
        const int h = (k != s);
        CK(cudaMemcpy((char*)(ctx->D.dyn + k) + off, &h, sizeof(int), cudaMemcpyHostToDevice));
    }
    const int rc = bs_prime(ctx);
    const int zero = 0;
    for (int k = 0; k < ctx->nscene; ++k)
        CK(cudaMemcpy((char*)(ctx->D.dyn + k) + off, &zero, sizeof(int), cudaMemcpyHostToDevice));
    return rc;
}

int bs_scalar_substep(bs_ctx* ctx) {
    if (!ctx) return BS_E_ARG;
    bs::disp(ctx->D, launch_of(ctx));
    st_scalar(ctx, 0);
    return check_launch(ctx);
}
int bs_projection(bs_ctx* ctx) {
    if (!ctx) return BS_E_ARG;
    bs::projection_only(ctx->D, launch_of(ctx));
    return check_launch(ctx);
}
int bs_cellshift(bs_ctx* ctx, int32_t alt) {
    if (!ctx) return BS_E_ARG;
    st_rebin(ctx, 0, alt ? 1 : 0);
    return check_launch(ctx);
}
int bs_search(bs_ctx* ctx) {
    if (!ctx) return BS_E_ARG;
    st_search(ctx, 1, 0);
    return check_launch(ctx);
}
int bs_porosity(bs_ctx* ctx) {
    if (!ctx) return BS_E_ARG;
    st_search(ctx, 0, 1);
    return check_launch(ctx);
}
int bs_eddy(bs_ctx* ctx) {
    if (!ctx) return BS_E_ARG;
    bs::eddy(ctx->D, launch_of(ctx), ctx->precision, 1, 0, 0);
    return check_launch(ctx);
}
int bs_int_vel(bs_ctx* ctx) {
    if (!ctx) return BS_E_ARG;
    bs::eddy(ctx->D, launch_of(ctx), ctx->precision, 0, 1, 0);   // varts (integrator.f90:468-507)
    bs::int_vel(ctx->D, launch_of(ctx), ctx->precision);
    return check_launch(ctx);
}
int bs_ppe_assemble(bs_ctx* ctx) {
    if (!ctx) return BS_E_ARG;
    bs::assemble(ctx->D, launch_of(ctx), ctx->precision);
    ctx->assembled = true;
    return check_launch(ctx);
}
int bs_ppe_solve(bs_ctx* ctx) {
    if (!ctx) return BS_E_ARG;
    if (!ctx->assembled) return fail(ctx, BS_E_STATE, "solve before assemble");
    int rc = st_solve(ctx);
    if (rc) return rc;
    rc = bs_sync(ctx);
    if (rc) return rc;
    unsigned e = 0;
    CK(cudaMemcpy(&e, ctx->D.err_word, sizeof(unsigned), cudaMemcpyDeviceToHost));
    if (e & BS_ERR_NOT_CONVERGED) return fail(ctx, BS_E_NOTCONV, "PPE solve did not converge");
    return 0;
}
int bs_comp_vel(bs_ctx* ctx) {
    if (!ctx) return BS_E_ARG;
    bs::comp_vel(ctx->D, launch_of(ctx), ctx->precision, 1, 0);
    bs::cell_max_timestep(ctx->D, launch_of(ctx), 1, 0);
    return check_launch(ctx);
}
int bs_comp_pos(bs_ctx* ctx) {
    if (!ctx) return BS_E_ARG;
    bs::comp_vel(ctx->D, launch_of(ctx), ctx->precision, 0, 1);
    return check_launch(ctx);
}
int bs_free_surface(bs_ctx* ctx) {
    if (!ctx) return BS_E_ARG;
    bs::freesurf(ctx->D, launch_of(ctx));
    return check_launch(ctx);
}
int bs_boun_vel(bs_ctx* ctx) {
    if (!ctx) return BS_E_ARG;
    bs::boun_vel(ctx->D, launch_of(ctx), ctx->precision);
    return check_launch(ctx);
}
int bs_ghost(bs_ctx* ctx, int32_t use_mls) {
    if (!ctx || (use_mls != 0 && use_mls != 1)) return BS_E_ARG;
    bs::ghost(ctx->D, launch_of(ctx), ctx->precision, use_mls);
    return check_launch(ctx);
}
int bs_collision_shift(bs_ctx* ctx, int32_t mode, double prx, double pry, double brx, double bry) {
    if (!ctx || (mode != 0 && mode != 1) || !(prx > 0) || !(pry > 0) || !(brx > 0) || !(bry > 0)) return BS_E_ARG;
    bs::collision_shift(ctx->D, launch_of(ctx), ctx->precision, mode, prx, pry, brx, bry);
    return check_launch(ctx);
}
int bs_shift(bs_ctx* ctx) {
    if (!ctx) return BS_E_ARG;
    bs::shift(ctx->D, launch_of(ctx), ctx->precision);
    bs::apply_density(ctx->D, launch_of(ctx), 1, 0);
    return check_launch(ctx);
}
int bs_density_update(bs_ctx* ctx) {
    if (!ctx) return BS_E_ARG;
    bs::apply_density(ctx->D, launch_of(ctx), 0, 1);
    return check_launch(ctx);
}
int bs_timestep(bs_ctx* ctx) {
    if (!ctx) return BS_E_ARG;
    bs::cell_max_timestep(ctx->D, launch_of(ctx), 0, 1);
    return check_launch(ctx);
}

// ---- WCSPH (wcsph.f90)
int bs_wcsph_continuity(bs_ctx* ctx) {
    if (!ctx) return BS_E_ARG;
    bs::wc_continuity(ctx->D, launch_of(ctx), ctx->precision);
    return check_launch(ctx);
}
int bs_wcsph_update_density(bs_ctx* ctx) {
    if (!ctx) return BS_E_ARG;
    bs::wc_rows(ctx->D, launch_of(ctx), 1);
    return check_launch(ctx);
}
int bs_wcsph_eos(bs_ctx* ctx) {
    if (!ctx) return BS_E_ARG;
    bs::wc_rows(ctx->D, launch_of(ctx), 2);
    return check_launch(ctx);
}
int bs_wcsph_pressure_to_density(bs_ctx* ctx) {
    if (!ctx) return BS_E_ARG;
    bs::wc_rows(ctx->D, launch_of(ctx), 4);
    return check_launch(ctx);
}
int bs_wcsph_wall_pressure(bs_ctx* ctx) {
    if (!ctx) return BS_E_ARG;
    bs::wc_wall_pressure(ctx->D, launch_of(ctx), ctx->precision);
    return check_launch(ctx);
}

// WCSPH step: bs_step's sequence with the PPE replaced by continuity,
// updateden, dentopress and the wall pressure; the porosity pass keeps the
// continuity density and densityupdate is left out.
int bs_wcsph_step(bs_ctx* ctx, int32_t nsteps) {
    if (!ctx || nsteps < 0) return BS_E_ARG;
    Dev& D = ctx->D;
    for (int it = 0; it < nsteps; ++it) {
        bs::Launch L = launch_of(ctx);
        if (ctx->any_zone)
            if (int rc = read_dyn(ctx)) return rc;
        bs::advance_time(D, L);
        bool any_scalar = false;
        for (auto& p : ctx->prm) any_scalar |= p.scalar_on != 0;
        if (any_scalar) {
            if (!ctx->disp_ready) {
                bs::disp(D, L);
                ctx->disp_ready = true;
            }
            for (int j1 = 0; j1 < ctx->max_solsteps; ++j1) st_scalar(ctx, j1);
        }
        if (int rc = st_buffers(ctx)) return rc;
        st_rebin(ctx, 1, 0);                 // projection + cellshift + resetid
        st_search(ctx, 1, 2);                // neighbour + effpor keeping the density
        bs::eddy(D, L, ctx->precision, 1, 1, 0);
        bs::int_vel(D, L, ctx->precision);
        bs::wc_continuity(D, L, ctx->precision);   // calmasscons
        bs::wc_rows(D, L, 1 | 2);            // updateden, dentopress
        bs::wc_wall_pressure(D, L, ctx->precision);
        bs::comp_vel(D, L, ctx->precision, 1, 1);   // comp_vel + comp_pos
        bs::cell_max_timestep(D, L, 1, 0);
        st_rebin(ctx, 0, 1);                 // cellshiftalt
        st_search(ctx, 1, 2);
        bs::freesurf(D, L);
        bs::shift(D, L, ctx->precision);
        bs::apply_density(D, L, 1, 0);       // shift apply only
        bs::cell_max_timestep(D, L, 0, 1);   // timestep
        bs::eddy(D, L, ctx->precision, 1, 0, 1);
        ctx->disp_ready = true;
        int rc = check_launch(ctx);
        if (rc) return rc;
        rc = read_solsteps(ctx);
        if (rc) return rc;
    }
    return 0;
}

// Full production step, main.f90:199-272 (open-boundary buffers excluded).
int bs_step(bs_ctx* ctx, int32_t nsteps) { return bs_step_flags(ctx, nsteps, BS_STEP_ALL); }

}  // extern "C"

// ------------------------------------------------------------ captured step
// A production step as one CUDA graph: the stages as stream capture on the
// context's stream, the salinity sub-steps and the Krylov loops as
// conditional while/if nodes whose condition kernels read the device's own
// counters (solsteps, converged scenes), so K steps are K graph launches
// with no host round trip.  The results are those of the eager step: the
// same kernels in the same order; the sub-steps run in pairs (the second of
// a pair beyond a scene's solsteps copies through, as the eager loop's
// surplus sub-steps do), which keeps the salinity buffers in place.
namespace {

bool any_scalar_on(const bs_ctx* ctx) {
    for (auto& p : ctx->prm)
        if (p.scalar_on) return true;
    return false;
}

int max_ppe_maxit(const bs_ctx* c) {
    int maxit = 0;
    for (auto& p : c->prm) maxit = std::max(maxit, (int)p.ppe_maxit);
    return maxit;
}

template <class T>
void key_put(std::vector<unsigned char>& k, const T& v) {
    const unsigned char* b = (const unsigned char*)&v;
    k.insert(k.end(), b, b + sizeof(T));
}

// everything the captured kernels and their launch shapes depend on
std::vector<unsigned char> step_key(const bs_ctx* c, int flags) {
    std::vector<unsigned char> k;
    key_put(k, c->D);
    const int v[] = {flags, c->precision, c->prm[0].ppe_solver, c->prm[0].ppe_restart, c->prm[0].ppe_precond,
                     c->prm[0].mixed_max_outer, max_ppe_maxit(c), c->mgsub_on, c->mgsub_level, c->mgsub_cs,
                     c->fg_df_on, c->disp_ready ? 1 : 0, any_scalar_on(c) ? 1 : 0, c->nblk_total,
                     c->sweep_tpb, c->mg0_tpb, c->mg_fp32, c->mgtail_level};
    key_put(k, v);
    for (const auto& m : c->mglev) key_put(k, m);
    k.insert(k.end(), c->mgneed.begin(), c->mgneed.end());
    return k;
}

// can this step be captured?  (buffer zones need the host's schedule, the
// per-kernel timer needs events between launches, and the FP32-inner
// refinement solver keeps its host loop)
bool step_graph_ok(const bs_ctx* c) {
    if (!c->step_graph_on || c->step_graph_broken || c->any_zone) return false;
    if (c->timer.mask) return false;
    const bool fg = c->prm[0].ppe_solver == BS_SOLVER_FGMRES;
    if (!fg && c->precision == BS_PREC_MIXED && c->prm[0].mixed_max_outer > 0) return false;
    return true;
}

// the stages of bs_step_flags, recorded into the capture of ctx->stream
bool record_step(bs_ctx* ctx, int flags) {
    Dev& D = ctx->D;
    bs::Launch L = launch_of(ctx);
    L.graph = nullptr;
    bs::advance_time(D, L);
    if (any_scalar_on(ctx) && (flags & BS_STEP_SCALAR)) {
        if (!ctx->disp_ready) {
            bs::disp(D, L);
            ctx->disp_ready = true;
        }
        cudaMemsetAsync(&D.loop->j, 0, sizeof(int), ctx->stream);
        cudaGraphConditionalHandle hs;
        if (!bs::cond_handle(ctx->stream, 1, &hs)) return false;
        const bool ok = bs::cond_node(ctx->stream, ctx->side[0], cudaGraphCondTypeWhile, hs, [&]() {
            bs::Launch B = L;
            B.stream = ctx->side[0];
            const int64_t b0 = ctx->launches;
            bs::scalar(D, B, ctx->precision, 0, &D.loop->j);   // sub-step j: con -> con_new
            std::swap(D.con, D.con_new);
            bs::scalar(D, B, ctx->precision, 1, &D.loop->j);   // sub-step j + 1: back into con
            std::swap(D.con, D.con_new);
            const int nk = (int)(ctx->launches - b0) + 1;
            bs::cond_scalar(D, ctx->side[0], hs, nk);
            ctx->launches = b0;
            return cudaGetLastError() == cudaSuccess;
        });
        if (!ok) return false;
    }
    if (flags & BS_STEP_BUFFERS)
        if (st_buffers(ctx)) return false;   // no zones here: nothing to do
    st_rebin(ctx, 1, 0);
    st_search(ctx, 1, 1);
    bs::eddy(D, L, ctx->precision, 1, 1, 0);
    bs::int_vel(D, L, ctx->precision);
    bs::assemble(D, L, ctx->precision);
    ctx->assembled = true;
    const int maxit = max_ppe_maxit(ctx);
    const int precond = ctx->prm[0].ppe_precond;
    bool ok;
    if (ctx->prm[0].ppe_solver == BS_SOLVER_FGMRES)
        ok = bs::capture_fgmres(D, L, ctx->side, maxit, precond ? 2 : 8, precond, mg_prec_of(ctx), ctx->d_nconv);
    else
        ok = bs::capture_fp64(D, L, ctx->side, maxit, precond ? 4 : 8, precond, mg_prec_of(ctx), ctx->d_nconv);
    if (!ok) return false;
    bs::comp_vel(D, L, ctx->precision, 1, 1);
    bs::cell_max_timestep(D, L, 1, 0);
    st_rebin(ctx, 0, 1);
    st_search(ctx, 1, 1);
    bs::freesurf(D, L);
    bs::shift(D, L, ctx->precision);
    bs::apply_density(D, L, 1, (flags & BS_STEP_DENSITY) ? 1 : 0);
    bs::cell_max_timestep(D, L, 0, 1);
    if (flags & BS_STEP_EDDY_END) {
        bs::eddy(D, L, ctx->precision, 1, 0, 1);
        ctx->disp_ready = true;
    } else {
        ctx->disp_ready = false;
    }
    return cudaGetLastError() == cudaSuccess;
}

// one step through the graph cache: 0 done, 1 not capturable (run eagerly),
// < 0 error
int step_graphed(bs_ctx* ctx, int flags) {
    if (ctx->prm[0].ppe_solver == BS_SOLVER_FGMRES) {
        if (int rc = fg_ensure(ctx)) return rc;   // allocations cannot happen inside a capture
        ctx->D.fg_df = (ctx->fg_df_on && ctx->precision == BS_PREC_MIXED && ctx->prm[0].ppe_precond) ? 1 : 0;
    }
    const std::vector<unsigned char> key = step_key(ctx, flags);
    bs_ctx::StepGraph* G = nullptr;
    for (auto& g : ctx->sgraphs)
        if (g.key == key) G = &g;
    if (!G) {
        const Dev D0 = ctx->D;
        const bool disp0 = ctx->disp_ready, asm0 = ctx->assembled;
        const int64_t l0 = ctx->launches;
        cudaGetLastError();
        cudaGraph_t gr = nullptr;
        cudaGraphExec_t ex = nullptr;
        bool ok = cudaStreamBeginCapture(ctx->stream, cudaStreamCaptureModeThreadLocal) == cudaSuccess;
        if (ok) {
            ok = record_step(ctx, flags);
            ok = (cudaStreamEndCapture(ctx->stream, &gr) == cudaSuccess) && ok && gr;
        }
        if (ok) ok = cudaGraphInstantiate(&ex, gr, 0) == cudaSuccess;
        if (gr) cudaGraphDestroy(gr);
        if (!ok) {   // put the host state back and step eagerly from now on
            if (ex) cudaGraphExecDestroy(ex);
            ctx->D = D0;
            ctx->disp_ready = disp0;
            ctx->assembled = asm0;
            ctx->launches = l0;
            ctx->step_graph_broken = true;
            cudaGetLastError();
            return 1;
        }
        if (ctx->sgraphs.size() >= 8) {   // drop the least recently used
            size_t o = 0;
            for (size_t i = 1; i < ctx->sgraphs.size(); ++i)
                if (ctx->sgraphs[i].used < ctx->sgraphs[o].used) o = i;
            cudaGraphExecDestroy(ctx->sgraphs[o].exec);
            ctx->sgraphs.erase(ctx->sgraphs.begin() + o);
        }
        bs_ctx::StepGraph g;
        g.exec = ex;
        g.key = key;
        g.after = ctx->D;
        g.disp_after = ctx->disp_ready;
        g.kernels = ctx->launches - l0;
        ctx->launches = l0;
        ctx->D = D0;
        ctx->sgraphs.push_back(std::move(g));
        G = &ctx->sgraphs.back();
    }
    G->used = ++ctx->sg_clock;
    CK(cudaGraphLaunch(G->exec, ctx->stream));
    ctx->D = G->after;
    ctx->disp_ready = G->disp_after;
    ctx->assembled = true;
    ctx->launches += G->kernels;
    ctx->graph_steps += 1;
    ctx->solsteps_stale = true;
    return check_launch(ctx);
}

}  // namespace

extern "C" {

// The production step of main.f90:199-272; the flags drop the parts the
// reference's settling phases (main.f90:39-67, 95-155) do not run.
int bs_step_flags(bs_ctx* ctx, int32_t nsteps, int32_t flags) {
    if (!ctx || nsteps < 0 || (flags & ~BS_STEP_ALL)) return BS_E_ARG;
    Dev& D = ctx->D;
    for (int it = 0; it < nsteps; ++it) {
        if (step_graph_ok(ctx)) {
            const int rc = step_graphed(ctx, flags);
            if (rc < 0) return rc;
            if (rc == 0) continue;
        }
        if (ctx->solsteps_stale) {   // the sub-step count of the last captured step
            if (int rc = read_solsteps(ctx)) return rc;
            ctx->solsteps_stale = false;
        }
        bs::Launch L = launch_of(ctx);
        if (ctx->any_zone)
            if (int rc = read_dyn(ctx)) return rc;
        bs::advance_time(D, L);
        bool any_scalar = false;
        for (auto& p : ctx->prm) any_scalar |= p.scalar_on != 0;
        if (any_scalar && (flags & BS_STEP_SCALAR)) {
            if (!ctx->disp_ready) {
                bs::disp(D, L);
                ctx->disp_ready = true;
            }
            // solsteps of the previous timestep() (read back at the end of the last step)
            for (int j1 = 0; j1 < ctx->max_solsteps; ++j1) st_scalar(ctx, j1);
        }
        if (flags & BS_STEP_BUFFERS)
            if (int rc = st_buffers(ctx)) return rc;   // remove_bufferN + insert_bufferN
        st_rebin(ctx, 1, 0);                 // projection + cellshift + resetid
        st_search(ctx, 1, 1);                // neighbour + effpor
        bs::eddy(D, L, ctx->precision, 1, 1, 0);  // eddyvis (+ varts of int_vel)
        bs::int_vel(D, L, ctx->precision);
        bs::assemble(D, L, ctx->precision);
        ctx->assembled = true;
        if (int rc = st_solve(ctx)) return rc;   // bicgstab / fgmres + pressure scatter
        bs::comp_vel(D, L, ctx->precision, 1, 1);   // comp_vel + comp_pos
        bs::cell_max_timestep(D, L, 1, 0);
        st_rebin(ctx, 0, 1);                 // cellshiftalt
        st_search(ctx, 1, 1);                // neighbour + effpor
        bs::freesurf(D, L);
        bs::shift(D, L, ctx->precision);     // opt2_shift
        bs::apply_density(D, L, 1, (flags & BS_STEP_DENSITY) ? 1 : 0);   // shift apply + densityupdate
        bs::cell_max_timestep(D, L, 0, 1);   // timestep
        if (flags & BS_STEP_EDDY_END) {
            bs::eddy(D, L, ctx->precision, 1, 0, 1);  // eddyvis (+ dispersion for the next scalar)
            ctx->disp_ready = true;
        } else {
            ctx->disp_ready = false;
        }
        int rc = check_launch(ctx);
        if (rc) return rc;
        rc = read_solsteps(ctx);   // next step's scalar sub-step count
        if (rc) return rc;
    }
    return 0;
}

// Overwrite fields of a scene in place, in the context's particle order
// (bs_download's): the host edits of the reference's driver between phases
// (main.f90:69-92, 156-191).  Non-NULL among vx, vy, p, mass, rho, oden,
// ovol, con; st->n must equal the scene's particle count.
int bs_set_fields(bs_ctx* ctx, int32_t s, const bs_state* st) {
    if (!ctx || s < 0 || s >= ctx->nscene || !st) return BS_E_ARG;
    CK(cudaStreamSynchronize(ctx->stream));
    Dev& D = ctx->D;
    SceneDyn hd;
    CK(cudaMemcpy(&hd, D.dyn + s, sizeof(hd), cudaMemcpyDeviceToHost));
    if (st->n != hd.n) return fail(ctx, BS_E_ARG, "bs_set_fields: particle count differs from the scene's");
    const size_t off = ctx->hpar[s].row0, n = hd.n;
    const double* src[] = {st->vx, st->vy, st->p, st->mass, st->rho, st->oden, st->ovol, st->con};
    double* dst[] = {D.vx, D.vy, D.p, D.mass, D.rho, D.oden, D.ovol, D.con};
    for (int f = 0; f < 8; ++f)
        if (src[f] && n) CK(cudaMemcpy(dst[f] + off, src[f], sizeof(double) * n, cudaMemcpyHostToDevice));
    bs::derive_fields(D, launch_of(ctx));   // vol = m/rho, nu from oden
    ctx->assembled = false;
    return check_launch(ctx);
}

// Set a scene's time (the reference restarts t at 0 for its production phase, main.f90:193-197)
int bs_set_time(bs_ctx* ctx, int32_t s, double t) {
    if (!ctx || s < 0 || s >= ctx->nscene) return BS_E_ARG;
    CK(cudaStreamSynchronize(ctx->stream));
    CK(cudaMemcpy(&ctx->D.dyn[s].t, &t, sizeof(double), cudaMemcpyHostToDevice));
    return 0;
}

// Stand-alone BiCGStab on a host CSR system: the system becomes a one-scene
// context (diagonal entries summed into adiag, the rest in the sliced ELL).
static int krylov_csr(int solver, int32_t n, const int32_t* row_ptr, const int32_t* col, const double* val,
                      const double* b, double* x, double tol, int32_t maxit, int32_t restart, int32_t stop_rule,
                      int32_t* iters, double* relres) {
    if (n <= 0 || !row_ptr || !col || !val || !b || !x) return BS_E_ARG;
    int kmax = 1;
    for (int r = 0; r < n; ++r) {
        int m = 0;
        for (int e = row_ptr[r]; e < row_ptr[r + 1]; ++e)
            if (col[e] != r) ++m;
        kmax = std::max(kmax, m);
    }
    if (kmax > 64) return BS_E_CAPACITY;
    bs_params p;
    bs_params_default(&p);
    p.cellx = p.celly = 4;
    p.kmax = kmax;
    p.ppe_tol = tol;
    p.ppe_maxit = maxit;
    p.ppe_stop = stop_rule;
    p.ppe_solver = solver;
    p.ppe_restart = restart;
    bs_ctx* ctx = nullptr;
    int rc = bs_create(1, &p, &n, nullptr, &ctx);
    if (rc) return rc;
    const ScenePar& P = ctx->hpar[0];
    const size_t E = (size_t)P.cap * kmax;
    std::vector<double> diag(n, 0.0), aval(E, 0.0);
    std::vector<int> idx(E, 0), cnt(n, 0);
    for (int r = 0; r < n; ++r)
        for (int e = row_ptr[r]; e < row_ptr[r + 1]; ++e) {
            if (col[e] == r) { diag[r] += val[e]; continue; }
            const size_t q = ((size_t)(r >> 5) * kmax + cnt[r]) * 32 + (r & 31);
            idx[q] = col[e];
            aval[q] = val[e];
            cnt[r]++;
        }
    Dev& D = ctx->D;
    SceneDyn hd;
    std::memset(&hd, 0, sizeof(hd));
    hd.n = n;
    CK(cudaMemcpy(D.dyn, &hd, sizeof(hd), cudaMemcpyHostToDevice));
    CK(cudaMemcpy(D.adiag, diag.data(), sizeof(double) * n, cudaMemcpyHostToDevice));
    CK(cudaMemcpy(D.rhs, b, sizeof(double) * n, cudaMemcpyHostToDevice));
    CK(cudaMemcpy(D.p, x, sizeof(double) * n, cudaMemcpyHostToDevice));
    CK(cudaMemcpy(D.ncount, cnt.data(), sizeof(int) * n, cudaMemcpyHostToDevice));
    CK(cudaMemcpy(D.nidx, idx.data(), sizeof(int) * E, cudaMemcpyHostToDevice));
    CK(cudaMemcpy(D.aval, aval.data(), sizeof(double) * E, cudaMemcpyHostToDevice));
    ctx->assembled = true;
    D.fg_df = 0;
    if (solver == BS_SOLVER_FGMRES)
        bs::solve_fgmres(D, launch_of(ctx), maxit, 1, 0, BS_PREC_FP64, ctx->d_nconv, ctx->h_pinned, ctx->evsync);
    else
        bs::solve_fp64(D, launch_of(ctx), maxit, 1, 0, BS_PREC_FP64, ctx->d_nconv, ctx->h_pinned, ctx->evsync);
    rc = bs_sync(ctx);
    if (!rc) {
        CK(cudaMemcpy(x, D.p, sizeof(double) * n, cudaMemcpyDeviceToHost));
        CK(cudaMemcpy(&hd, D.dyn, sizeof(hd), cudaMemcpyDeviceToHost));
        if (iters) *iters = hd.iters;
        if (relres) *relres = hd.relres;
        if (hd.err & BS_ERR_NOT_CONVERGED) rc = BS_E_NOTCONV;
    }
    bs_destroy(ctx);
    return rc;
}

int bs_bicgstab_csr(int32_t n, const int32_t* row_ptr, const int32_t* col, const double* val, const double* b,
                    double* x, double tol, int32_t maxit, int32_t stop_rule, int32_t* iters, double* relres) {
    return krylov_csr(BS_SOLVER_BICGSTAB, n, row_ptr, col, val, b, x, tol, maxit, 150, stop_rule, iters, relres);
}

int bs_fgmres_csr(int32_t n, const int32_t* row_ptr, const int32_t* col, const double* val, const double* b,
                  double* x, double tol, int32_t maxit, int32_t restart, int32_t stop_rule, int32_t* iters,
                  double* relres) {
    if (restart < 1 || restart > BS_FG_MAXM) return BS_E_ARG;
    return krylov_csr(BS_SOLVER_FGMRES, n, row_ptr, col, val, b, x, tol, maxit, restart, stop_rule, iters, relres);
}

int bs_event_record(bs_ctx* ctx, int32_t slot) {
    if (!ctx || slot < 0 || slot >= 16) return BS_E_ARG;
    CK(cudaEventRecord(ctx->ev[slot], ctx->stream));
    return 0;
}
int bs_event_elapsed_ms(bs_ctx* ctx, int32_t a, int32_t b, float* ms) {
    if (!ctx || a < 0 || a >= 16 || b < 0 || b >= 16 || !ms) return BS_E_ARG;
    CK(cudaEventSynchronize(ctx->ev[b]));
    CK(cudaEventElapsedTime(ms, ctx->ev[a], ctx->ev[b]));
    return 0;
}
// enable: bit mask of kernel ids to bracket with events (0 disables); resets totals
int bs_kernel_timing(bs_ctx* ctx, uint64_t enable) {
    if (!ctx) return BS_E_ARG;
    CK(cudaStreamSynchronize(ctx->stream));
    bs::KTimer& T = ctx->timer;
    if (!T.ready && enable) {
        for (int q = 0; q < bs::KTimer::NEV; ++q) CK(cudaEventCreate(&T.ev[q]));
        T.ready = true;
    }
    bs::timer_collect(&T, true);
    T.mask = (unsigned long long)enable;
    for (int k = 0; k < bs::K_COUNT; ++k) {
        T.total_ms[k] = 0.0;
        T.count[k] = 0;
    }
    return 0;
}
int bs_kernel_timing_get(bs_ctx* ctx, int32_t idx, const char** name, int32_t* launches, double* total_ms) {
    if (!ctx || idx < 0 || idx >= bs::K_COUNT) return BS_E_ARG;
    CK(cudaStreamSynchronize(ctx->stream));
    bs::timer_collect(&ctx->timer, true);
    if (name) *name = bs::kernel_names[idx];
    if (launches) *launches = (int32_t)ctx->timer.count[idx];
    if (total_ms) *total_ms = ctx->timer.total_ms[idx];
    return 0;
}
int64_t bs_launch_count(bs_ctx* ctx) {
    if (!ctx) return -1;
    int64_t n = ctx->launches;
    if (ctx->graph_steps) {   // kernels of the captured steps' device loops, counted on the device
        unsigned long long k = 0;
        if (cudaStreamSynchronize(ctx->stream) != cudaSuccess ||
            cudaMemcpy(&k, &ctx->D.loop->kernels, sizeof(k), cudaMemcpyDeviceToHost) != cudaSuccess)
            return -1;
        n += (int64_t)k;
    }
    return n;
}

int bs_device_memory(size_t* free_bytes, size_t* total_bytes) {
    if (!free_bytes || !total_bytes) return BS_E_ARG;
    return cudaMemGetInfo(free_bytes, total_bytes) == cudaSuccess ? BS_OK : BS_E_CUDA;
}

int bs_context_bytes(bs_ctx* ctx, size_t* bytes) {
    if (!ctx || !bytes) return BS_E_ARG;
    size_t t = 0;
    for (size_t b : ctx->alloc_bytes) t += b;
    *bytes = t;
    return BS_OK;
}

}  // extern "C"
