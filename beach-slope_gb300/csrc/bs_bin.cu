// bs_bin.cu -- cell re-binning by counting sort (cellshift / cellshiftalt /
// resetid, integrator.f90:33-392, isph.f90:88-113), plus projection,
// per-cell maxima and the timestep rule.
//
// The reference moves each fluid particle to one of its cell's 8 neighbours
// by half-open comparisons against the cell bounds and rebuilds every cell's
// list as [walls][stayers in slot order][arrivals from (i+1,j), (i-1,j),
// (i,j+1), (i,j-1), (i-1,j-1), (i+1,j-1), (i-1,j+1), (i+1,j+1), each in the
// source cell's slot order].  That order is a stable sort by the key
// (destination cell, arrival category) over rows that are already sorted by
// source cell, so a counting sort over BS_NCAT buckets per cell reproduces
// it exactly:  k_rank (one warp per source cell: codes + ballot ranks +
// bucket counts) -> k_scan_part (per cell: prefix over its buckets; per
// chunk of cells: the total) -> k_scan_apply (per scene: exclusive scan of
// the cell totals) -> k_permute.
#include "bs_internal.cuh"

namespace {

// arrival category = code; destination key offset for each code
// 0 wall, 1 stay, 2 moved north (tn, to i-1), 3 south (ts, i+1), 4 west (tw,
// j-1), 5 east (te, j+1), 6 south-east (tse, i+1,j+1), 7 north-east (tne,
// i-1,j+1), 8 south-west (tsw, i+1,j-1), 9 north-west (tnw, i-1,j-1), 10 lost
__device__ __forceinline__ void code_di_dj(int code, int& di, int& dj) {
    const int tdi[10] = {0, 0, -1, 1, 0, 0, 1, -1, 1, -1};
    const int tdj[10] = {0, 0, 0, 0, -1, 1, 1, 1, -1, -1};
    di = tdi[code];
    dj = tdj[code];
}

__device__ __forceinline__ int classify(const ScenePar& P, int i, int j, double x1, double y1) {
    const double xl = cell_xleft(P, j), xr = cell_xright(P, j);
    const double yb = cell_ybot(P, i), yt = cell_ytop(P, i);
    if ((x1 >= xl) && (x1 < xr)) {
        if ((y1 >= yb) && (y1 < yt)) return 1;
        if (y1 < yb) return 3;
        if (y1 >= yt) return 2;
    } else if (x1 >= xr) {
        if (y1 >= yt) return 7;
        if ((y1 >= yb) && (y1 < yt)) return 5;
        if (y1 < yb) return 6;
    } else if (x1 < xl) {
        if (y1 >= yt) return 9;
        if ((y1 >= yb) && (y1 < yt)) return 4;
        if (y1 < yb) return 8;
    }
    return 10;
}

// projection, isph.f90:17-47: x = x + (dt*vx/porosity), written without FMA
__device__ __forceinline__ double project(double x, double dt, double v, double por) {
    return __dadd_rn(x, __ddiv_rn(__dmul_rn(dt, v), por));
}

__global__ void k_rank(Dev D, int projection, int cutoff) {
    const int warp = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const int lane = threadIdx.x & 31;
    if (warp >= D.ncell_total) return;
    const int c = warp;
    const int s = D.cell_scene[c];
    const ScenePar& P = D.par[s];
    const int lc = c - P.cell0;
    const int i = lc % P.celly + 1, j = lc / P.celly + 1;
    const int r0 = D.cell_start[c], r1 = D.cell_end[c];
    int cnt[11];
#pragma unroll
    for (int d = 0; d < 11; ++d) cnt[d] = 0;
    const double dt = D.dyn[s].dt;
    const unsigned lt = (1u << lane) - 1u;
    for (int base = r0; base < r1; base += 32) {
        const int r = base + lane;
        int code = 11;   // inactive lane
        if (r < r1) {
            if (D.tid[r] != BS_TID_FLUID) {
                code = 0;
            } else {
                double x1 = D.x[r], y1 = D.y[r];
                if (projection) {
                    const double por = D.por[r];
                    x1 = project(x1, dt, D.vx[r], por);
                    y1 = project(y1, dt, D.vy[r], por);
                }
                code = classify(P, i, j, x1, y1);
                if (cutoff && code != 10) {   // integrator.f90:61-62
                    const bool buf = D.flags[r] & BS_FLAG_BUFFER;
                    const bool keep = (x1 > P.xlcutoff) || buf || ((x1 <= P.xlcutoff) && (y1 <= P.ytcutoff));
                    if (!keep) code = 10;
                }
                if (code >= 2 && code <= 9) {   // destination must be an interior cell
                    int di, dj;
                    code_di_dj(code, di, dj);
                    const int ii = i + di, jj = j + dj;
                    if (ii < 2 || ii > P.celly - 1 || jj < 2 || jj > P.cellx - 1) code = 10;
                }
            }
        }
#pragma unroll
        for (int d = 0; d < 11; ++d) {
            const unsigned m = __ballot_sync(0xffffffffu, code == d);
            if (code == d) D.coderank[r] = (d << 24) | (cnt[d] + __popc(m & lt));
            cnt[d] += __popc(m);
        }
    }
    if (lane < 10) {
        int di, dj;
        code_di_dj(lane, di, dj);
        const int ii = i + di, jj = j + dj;
        if (ii >= 2 && ii <= P.celly - 1 && jj >= 2 && jj <= P.cellx - 1) {
            int v = 0;
#pragma unroll
            for (int d = 0; d < 10; ++d)
                if (d == lane) v = cnt[d];
            if (v) D.bucket[(long)(c + di + dj * P.celly) * BS_NCAT + lane] = v;
        }
    }
    if (lane == 0 && cnt[10] > 0) {
        atomicAdd(&D.dyn[s].lost, cnt[10]);
        if (!cutoff) set_err(D, s, BS_ERR_LOST_PARTICLE);
    }
}

// Per-scene exclusive scan of the cell totals in two passes over chunks of
// BS_SCAN_CHUNK cells, block (k, s) = chunk k of scene s.  Pass 1: each
// cell's prefix over its buckets (the rows of each category before it) and
// its total, and the chunk's total.
__global__ void __launch_bounds__(BS_SCAN_CHUNK) k_scan_part(Dev D) {
    const int s = blockIdx.y, k = blockIdx.x;
    const ScenePar& P = D.par[s];
    if (k * BS_SCAN_CHUNK >= P.ncell) return;
    __shared__ int ws[BS_SCAN_CHUNK / 32];
    const int q = k * BS_SCAN_CHUNK + threadIdx.x, lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    int acc = 0;
    if (q < P.ncell) {
        int* b = D.bucket + (long)(P.cell0 + q) * BS_NCAT;
#pragma unroll
        for (int d = 0; d < BS_NCAT; ++d) {
            const int v = b[d];
            b[d] = acc;
            acc += v;
        }
        D.cell_total[P.cell0 + q] = acc;
    }
    int v = acc;
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    if (lane == 0) ws[w] = v;
    __syncthreads();
    if (w == 0) {
        int a = ws[lane];
        for (int o = 16; o > 0; o >>= 1) a += __shfl_xor_sync(0xffffffffu, a, o);
        if (lane == 0) D.scan_part[s * D.scan_chunks + k] = a;
    }
}

// Pass 2: the chunk's exclusive scan, offset by the totals of the scene's
// chunks before it, as the cells' row ranges in the permuted order; the
// scene's last chunk records the new particle count.
__global__ void __launch_bounds__(BS_SCAN_CHUNK) k_scan_apply(Dev D) {
    const int s = blockIdx.y, k = blockIdx.x;
    const ScenePar& P = D.par[s];
    if (k * BS_SCAN_CHUNK >= P.ncell) return;
    __shared__ int ws[BS_SCAN_CHUNK / 32];
    __shared__ int base;
    const int q = k * BS_SCAN_CHUNK + threadIdx.x, lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    if (w == 0) {
        int a = 0;
        for (int i = lane; i < k; i += 32) a += D.scan_part[s * D.scan_chunks + i];
        for (int o = 16; o > 0; o >>= 1) a += __shfl_xor_sync(0xffffffffu, a, o);
        if (lane == 0) base = a;
    }
    const int v = q < P.ncell ? D.cell_total[P.cell0 + q] : 0;
    int inc = v;   // inclusive scan within the warp
    for (int o = 1; o < 32; o <<= 1) {
        const int u = __shfl_up_sync(0xffffffffu, inc, o);
        if (lane >= o) inc += u;
    }
    if (lane == 31) ws[w] = inc;
    __syncthreads();
    if (w == 0) {
        int x = ws[lane];
        for (int o = 1; o < 32; o <<= 1) {
            const int u = __shfl_up_sync(0xffffffffu, x, o);
            if (lane >= o) x += u;
        }
        ws[lane] = x;   // inclusive warp prefix
    }
    __syncthreads();
    if (q < P.ncell) {
        const int start = P.row0 + base + (w ? ws[w - 1] : 0) + inc - v;
        D.cell_start2[P.cell0 + q] = start;
        D.cell_end2[P.cell0 + q] = start + v;
    }
    if (threadIdx.x == 0 && (k + 1) * BS_SCAN_CHUNK >= P.ncell) {
        D.dyn[s].n_prev = D.dyn[s].n;
        D.dyn[s].n = base + ws[BS_SCAN_CHUNK / 32 - 1];
    }
}

__global__ void k_permute(Dev D, int projection) {
    const int r = blockIdx.x * blockDim.x + threadIdx.x;
    const int s = D.blk_scene[blockIdx.x];
    const ScenePar& P = D.par[s];
    if (r >= P.row0 + D.dyn[s].n_prev) return;
    const int cr = D.coderank[r];
    const int code = cr >> 24, rank = cr & 0xffffff;
    if (code >= 10) return;
    const int c = D.cell[r];
    int di, dj;
    code_di_dj(code, di, dj);
    const int dc = c + di + dj * P.celly;
    const int dr = D.cell_start2[dc] + D.bucket[(long)dc * BS_NCAT + code] + rank;
    double x = D.x[r], y = D.y[r], xs = D.xs[r], ys = D.ys[r];
    if (projection && D.tid[r] == BS_TID_FLUID) {
        const double dt = D.dyn[s].dt, por = D.por[r];
        xs = x;
        ys = y;
        x = project(x, dt, D.vx[r], por);
        y = project(y, dt, D.vy[r], por);
    }
    D.x2[dr] = x; D.y2[dr] = y; D.xs2[dr] = xs; D.ys2[dr] = ys;
    D.vx2[dr] = D.vx[r]; D.vy2[dr] = D.vy[r]; D.vxs2[dr] = D.vxs[r]; D.vys2[dr] = D.vys[r];
    D.p2[dr] = D.p[r]; D.mass2[dr] = D.mass[r]; D.rho2[dr] = D.rho[r]; D.oden2[dr] = D.oden[r];
    D.ovol2[dr] = D.ovol[r]; D.con2[dr] = D.con[r]; D.vol2[dr] = D.vol[r]; D.nu2[dr] = D.nu[r];
    D.tid2[dr] = D.tid[r]; D.flags2[dr] = D.flags[r]; D.pid2[dr] = D.pid[r]; D.cell2[dr] = dc;
}

// projection alone (isph.f90:17-47), for the per-stage entry point
__global__ void k_projection(Dev D) {
    const int r = blockIdx.x * blockDim.x + threadIdx.x;
    const int s = D.blk_scene[blockIdx.x];
    const ScenePar& P = D.par[s];
    if (r >= P.row0 + D.dyn[s].n || D.tid[r] != BS_TID_FLUID) return;
    const double dt = D.dyn[s].dt, por = D.por[r];
    const double x = D.x[r], y = D.y[r];
    D.xs[r] = x;
    D.ys[r] = y;
    D.x[r] = project(x, dt, D.vx[r], por);
    D.y[r] = project(y, dt, D.vy[r], por);
}

// Per-cell maxima of |vel| and |nut| (integrator.f90:831-841; an empty cell
// keeps its old values) and the timestep rule (integrator.f90:885-953).
// One thread per cell; per-scene finisher = last block of the scene.
__global__ void k_cellmax(Dev D, int do_cellmax) {
    const int c = blockIdx.x * blockDim.x + threadIdx.x;
    if (c >= D.ncell_total || !do_cellmax || D.dyn[D.cell_scene[c]].hold) return;
    const int r0 = D.cell_start[c], r1 = D.cell_end[c];
    if (r1 > r0) {
        double mv = 0.0, me = 0.0;
        for (int r = r0; r < r1; ++r) {
            mv = fmax(mv, fabs(D.vel[r]));
            me = fmax(me, fabs(D.nut[r]));
        }
        D.cell_maxvel[c] = mv;
        D.cell_maxeddy[c] = me;
    }
}

// Per-scene maxima over the interior cells of the cell maxima (k_cellmax)
// for the timestep rule (integrator.f90:885-953): one thread per cell, a
// segmented warp maximum over the warp's cells of one scene, one atomic
// maximum per segment on the bit patterns (non-negative doubles order as
// unsigned integers).  A value that is not positive counts as 0, as in the
// rule's running fmax from 0, which passes over NaN.
__global__ void k_scene_max(Dev D) {
    const int c = blockIdx.x * blockDim.x + threadIdx.x;
    const int lane = threadIdx.x & 31;
    int s = -1;
    unsigned long long v0 = 0ull, v1 = 0ull;
    if (c < D.ncell_total) {
        s = D.cell_scene[c];
        const ScenePar& P = D.par[s];
        const int lc = c - P.cell0;
        const int i = lc % P.celly + 1, j = lc / P.celly + 1;
        if (!D.dyn[s].hold && i >= 2 && i <= P.celly - 1 && j >= 2 && j <= P.cellx - 1) {
            const double a = D.cell_maxvel[c], b = D.cell_maxeddy[c];
            v0 = a > 0.0 ? (unsigned long long)__double_as_longlong(a) : 0ull;
            v1 = b > 0.0 ? (unsigned long long)__double_as_longlong(b) : 0ull;
        }
    }
    for (int o = 1; o < 32; o <<= 1) {   // cells of one scene are contiguous
        const unsigned long long a = __shfl_down_sync(0xffffffffu, v0, o), b = __shfl_down_sync(0xffffffffu, v1, o);
        const int so = __shfl_down_sync(0xffffffffu, s, o);
        if (lane + o < 32 && so == s) {
            v0 = a > v0 ? a : v0;
            v1 = b > v1 ? b : v1;
        }
    }
    const int sp = __shfl_up_sync(0xffffffffu, s, 1);
    if (s >= 0 && (lane == 0 || sp != s)) {
        if (v0) atomicMax(D.scene_max + 2 * s, v0);
        if (v1) atomicMax(D.scene_max + 2 * s + 1, v1);
    }
}

// the timestep rule per scene from the maxima of k_scene_max (which it
// clears for the next step)
__global__ void k_timestep(Dev D) {
    const int s = blockIdx.x * blockDim.x + threadIdx.x;
    if (s >= D.nscene) return;
    unsigned long long* m = D.scene_max + 2 * s;
    const double umax = __longlong_as_double((long long)m[0]);
    double numax = __longlong_as_double((long long)m[1]);
    m[0] = 0ull;
    m[1] = 0ull;
    if (D.dyn[s].hold) return;
    const ScenePar& P = D.par[s];
    {
        SceneDyn& Y = D.dyn[s];
        Y.umax = umax;
        const double sig1 = P.sig1, dl = P.dl, mu = P.mu, rho = P.rho, t = Y.t;
        double dt = Y.dt;
        if (P.adaptive_dt) {
            if (t <= 1.0)
                dt = fmin(fmin(sig1 * (dl) / umax, sig1 * ((dl) * (dl)) / ((mu / rho) + numax)), 0.0010);
            else if ((t > 1.0) && (t <= 2.50))
                dt = (double)fminf(fminf((float)(sig1 * (dl) / umax), (float)(sig1 * ((dl) * (dl)) * rho / mu)), 0.002f);
            else if ((t > 3.0) && (t <= 4.0))
                dt = (double)fminf(fminf((float)(sig1 * (dl) / umax), (float)(sig1 * ((dl) * (dl)) * rho / mu)), 0.004f);
            else
                dt = fmin(fmin(sig1 * (dl) / umax, sig1 * ((dl) * (dl)) / ((mu / rho) + numax)), 0.0050);
            Y.dt = dt;
        }
        if (!isfinite(numax)) numax = 0.0;
        Y.numax = numax;
        double dtsol = sig1 * (dl * dl) / (BS_SP1EM9 + numax / P.tschmidt);
        int solsteps = 1;
        if (dtsol < dt) {
            solsteps = (int)ceil(dt / dtsol);
            dtsol = dt / solsteps;
        }
        dtsol = (dtsol < dt) ? dtsol : dt;
        Y.dtsol = dtsol;
        Y.solsteps = solsteps;
    }
}

__global__ void k_advance_time(Dev D) {
    const int s = blockIdx.x * blockDim.x + threadIdx.x;
    if (s < D.nscene) D.dyn[s].t = D.dyn[s].t + D.dyn[s].dt;
}

// A scene's upload, placed: the caller copied the host's arrays in input
// order into the alternate particle buffers (x2 ... con2, tid2, flags2,
// pid2), each particle's bucket (2 cell + fluid) into cell2 and, into
// coderank, the input index of every binned row (the host's stable counting
// sort by cell, walls first, input order: boundary.f90:140-190,
// internal.f90:73-95).  Row r gathers its particle and sets the fields the
// upload starts from: xs = x, ys = y, vxs = vys = 0, porosity 1.
__global__ void k_upload_gather(Dev D, int row0, int n, int cell0, int has_flags, int has_pid) {
    const int q = blockIdx.x * blockDim.x + threadIdx.x;
    if (q >= n) return;
    const int i = D.coderank[row0 + q];
    const int r = row0 + q, g = row0 + i;
    const double x = D.x2[g], y = D.y2[g];
    D.x[r] = x;
    D.y[r] = y;
    D.xs[r] = x;
    D.ys[r] = y;
    D.vx[r] = D.vx2[g];
    D.vy[r] = D.vy2[g];
    D.p[r] = D.p2[g];
    D.mass[r] = D.mass2[g];
    D.rho[r] = D.rho2[g];
    D.oden[r] = D.oden2[g];
    D.ovol[r] = D.ovol2[g];
    D.con[r] = D.con2[g];
    D.vxs[r] = 0.0;
    D.vys[r] = 0.0;
    D.por[r] = 1.0;
    D.tid[r] = D.tid2[g];
    D.flags[r] = has_flags ? D.flags2[g] : (uint8_t)0;
    D.pid[r] = has_pid ? D.pid2[g] : i + 1;
    D.cell[r] = D.cell2[g] / 2 + cell0;
}

// Rows [row0, row0 + n) of the requested fields into the snapshot buffer
// (same row positions), one launch in stream order after a step: the copy
// to the host then reads the snapshot while the next steps run.
__global__ void k_snapshot(const __grid_constant__ bs::SnapArgs a) {
    const int q = blockIdx.x * blockDim.x + threadIdx.x;
    if (q >= a.n) return;
    const int r = a.row0 + q;
    for (int f = 0; f < a.nf; ++f) a.dst[f][r] = a.src[f][r];
    if (a.tid) a.tid_dst[r] = a.tid[r];
    if (a.pid) a.pid_dst[r] = a.pid[r];
    if (a.flags) a.flags_dst[r] = a.flags[r];
}

// derived per-particle fields after upload / density update
__global__ void k_derive(Dev D) {
    const int r = blockIdx.x * blockDim.x + threadIdx.x;
    const int s = D.blk_scene[blockIdx.x];
    const ScenePar& P = D.par[s];
    if (r >= P.row0 + D.dyn[s].n) return;
    D.vol[r] = D.mass[r] / D.rho[r];
    const double od = D.oden[r];
    D.nu[r] = (D.tid[r] == BS_TID_FLUID) ? bs_vis(od) / od : 0.0;
}

// ------------------------------------------------- open-boundary buffers
// remove_bufferN + insert_bufferN (internal.f90:447-586) on one scene: the
// zone's entry cells lose their buffer particles at or beyond remove_x (the
// others keep their order) and gain the template particles inside them, in
// template order, after the survivors.  Other cells keep their rows.  The
// reference compacts plist but not the per-slot pplist, so the porosity that
// the next projection reads is the one of the cell's slot position: new slot
// k takes the porosity of old slot k, and a slot beyond the cell's old count
// the properties' default, 1 (particle.f90:60-69).

__device__ __forceinline__ bool bx_removed(const bs::ZoneDev& Z, double x, uint8_t fl) {
    if (!(fl & BS_FLAG_BUFFER)) return false;
    return Z.remove_side > 0 ? (x >= Z.remove_x) : (x <= Z.remove_x);
}

// one warp per cell of scene s: new cell total; old range kept in cell_start2/end2
__global__ void k_bx_count(Dev D, int s, bs::ZoneDev Z) {
    const ScenePar& P = D.par[s];
    const int warp = (blockIdx.x * blockDim.x + threadIdx.x) >> 5, lane = threadIdx.x & 31;
    if (warp >= P.ncell) return;
    const int c = P.cell0 + warp;
    const int r0 = D.cell_start[c], r1 = D.cell_end[c];
    int keep = r1 - r0, add = 0;
    if (D.czone[c] & (1u << Z.zone)) {
        keep = 0;
        for (int base = r0; base < r1; base += 32) {
            const int r = base + lane;
            const bool k = (r < r1) && !bx_removed(Z, D.x[r], D.flags[r]);
            keep += __popc(__ballot_sync(0xffffffffu, k));
        }
        add = D.zcount[Z.zone][c];
    }
    if (lane == 0) {
        D.cell_start2[c] = r0;
        D.cell_end2[c] = r1;
        D.cell_total[c] = keep + add;
        D.bucket[(long)c * BS_NCAT] = keep;
    }
}

// the scene's rows (and porosity) into the alternate buffers
__global__ void k_bx_copyout(Dev D, int s) {
    const ScenePar& P = D.par[s];
    const int r = P.row0 + blockIdx.x * blockDim.x + threadIdx.x;
    if (r >= P.row0 + D.dyn[s].n) return;
    D.x2[r] = D.x[r]; D.y2[r] = D.y[r]; D.xs2[r] = D.xs[r]; D.ys2[r] = D.ys[r];
    D.vx2[r] = D.vx[r]; D.vy2[r] = D.vy[r]; D.vxs2[r] = D.vxs[r]; D.vys2[r] = D.vys[r];
    D.p2[r] = D.p[r]; D.mass2[r] = D.mass[r]; D.rho2[r] = D.rho[r]; D.oden2[r] = D.oden[r];
    D.ovol2[r] = D.ovol[r]; D.con2[r] = D.con[r]; D.vol2[r] = D.vol[r]; D.nu2[r] = D.nu[r];
    D.tid2[r] = D.tid[r]; D.flags2[r] = D.flags[r]; D.pid2[r] = D.pid[r];
    D.sxd[r] = D.por[r];
}

// one block: exclusive scan of the scene's new cell totals -> cell_start/end, n
__global__ void k_bx_scan(Dev D, int s) {
    const ScenePar& P = D.par[s];
    __shared__ int sh[1024];
    __shared__ int carry;
    if (threadIdx.x == 0) carry = 0;
    __syncthreads();
    const int nb = blockDim.x;
    for (int base = 0; base < P.ncell; base += nb) {
        const int q = base + threadIdx.x;
        const int v = (q < P.ncell) ? D.cell_total[P.cell0 + q] : 0;
        sh[threadIdx.x] = v;
        __syncthreads();
        for (int o = 1; o < nb; o <<= 1) {
            const int t = (threadIdx.x >= o) ? sh[threadIdx.x - o] : 0;
            __syncthreads();
            sh[threadIdx.x] += t;
            __syncthreads();
        }
        if (q < P.ncell) {
            const int st = P.row0 + carry + sh[threadIdx.x] - v;
            D.cell_start[P.cell0 + q] = st;
            D.cell_end[P.cell0 + q] = st + v;
        }
        __syncthreads();
        if (threadIdx.x == nb - 1) carry += sh[nb - 1];
        __syncthreads();
    }
    if (threadIdx.x == 0) D.dyn[s].n = carry;
}

// one warp per cell: survivors (stable) then the cell's template particles
__global__ void k_bx_scatter(Dev D, int s, bs::ZoneDev Z) {
    const ScenePar& P = D.par[s];
    const int warp = (blockIdx.x * blockDim.x + threadIdx.x) >> 5, lane = threadIdx.x & 31;
    if (warp >= P.ncell) return;
    const int c = P.cell0 + warp;
    const int o0 = D.cell_start2[c], o1 = D.cell_end2[c];
    const int oldn = o1 - o0;
    const int n0 = D.cell_start[c];
    const bool zc = D.czone[c] & (1u << Z.zone);
    const unsigned lt = (1u << lane) - 1u;
    int kept = 0;
    for (int base = o0; base < o1; base += 32) {
        const int r = base + lane;
        const bool k = (r < o1) && !(zc && bx_removed(Z, D.x2[r], D.flags2[r]));
        const unsigned m = __ballot_sync(0xffffffffu, k);
        if (k) {
            const int slot = kept + __popc(m & lt);
            const int d = n0 + slot;
            D.x[d] = D.x2[r]; D.y[d] = D.y2[r]; D.xs[d] = D.xs2[r]; D.ys[d] = D.ys2[r];
            D.vx[d] = D.vx2[r]; D.vy[d] = D.vy2[r]; D.vxs[d] = D.vxs2[r]; D.vys[d] = D.vys2[r];
            D.p[d] = D.p2[r]; D.mass[d] = D.mass2[r]; D.rho[d] = D.rho2[r]; D.oden[d] = D.oden2[r];
            D.ovol[d] = D.ovol2[r]; D.con[d] = D.con2[r]; D.vol[d] = D.vol2[r]; D.nu[d] = D.nu2[r];
            D.tid[d] = D.tid2[r]; D.flags[d] = D.flags2[r]; D.pid[d] = D.pid2[r]; D.cell[d] = c;
            D.por[d] = D.sxd[o0 + slot];   // slot position (slot < old count here)
        }
        kept += __popc(m);
    }
    if (!zc) return;
    const int t0 = D.zstart[Z.zone][c], tn = D.zcount[Z.zone][c];
    for (int q = lane; q < tn; q += 32) {
        const int t = t0 + q;
        const int slot = kept + q;
        const int d = n0 + slot;
        D.x[d] = Z.x[t]; D.y[d] = Z.y[t]; D.xs[d] = 0.0; D.ys[d] = 0.0;
        D.vx[d] = Z.vx[t]; D.vy[d] = Z.vy[t]; D.vxs[d] = 0.0; D.vys[d] = 0.0;
        D.p[d] = Z.p[t]; D.mass[d] = Z.mass; D.rho[d] = Z.rho; D.oden[d] = Z.rho;
        D.ovol[d] = Z.ovol; D.con[d] = Z.con;
        D.vol[d] = Z.mass / Z.rho;
        D.nu[d] = bs_vis(Z.rho) / Z.rho;
        D.tid[d] = BS_TID_FLUID; D.flags[d] = BS_FLAG_BUFFER; D.pid[d] = Z.pid ? Z.pid[t] : 0; D.cell[d] = c;
        D.por[d] = (slot < oldn) ? D.sxd[o0 + slot] : 1.0;
    }
}

inline unsigned gdiv(long a, int b) { return (unsigned)((a + b - 1) / b); }

}  // namespace

namespace bs {

void rebin(const Dev& D, const Launch& L, int projection, int cutoff) {
    cudaMemsetAsync(D.bucket, 0, sizeof(int) * (size_t)D.ncell_total * BS_NCAT, L.stream);
    int q = tbegin(L, K_RANK);
    k_rank<<<gdiv((long)D.ncell_total * 32, BS_THREADS), BS_THREADS, 0, L.stream>>>(D, projection, cutoff);
    tend(L, q);
    q = tbegin(L, K_CELLPREFIX);
    k_scan_part<<<dim3(D.scan_chunks, D.nscene), BS_SCAN_CHUNK, 0, L.stream>>>(D);
    tend(L, q);
    q = tbegin(L, K_SCANCELLS);
    k_scan_apply<<<dim3(D.scan_chunks, D.nscene), BS_SCAN_CHUNK, 0, L.stream>>>(D);
    tend(L, q);
    q = tbegin(L, K_PERMUTE);
    k_permute<<<L.nblk_rows, BS_THREADS, 0, L.stream>>>(D, projection);
    tend(L, q);
}

void buffer_exchange(const Dev& D, const Launch& L, int s, const ScenePar& P, const ZoneDev& Z) {
    const int q = tbegin(L, K_BUFX);
    const unsigned gc = gdiv((long)P.ncell * 32, BS_THREADS);
    k_bx_count<<<gc, BS_THREADS, 0, L.stream>>>(D, s, Z);
    k_bx_copyout<<<P.nblk, BS_THREADS, 0, L.stream>>>(D, s);
    k_bx_scan<<<1, 1024, 0, L.stream>>>(D, s);
    k_bx_scatter<<<gc, BS_THREADS, 0, L.stream>>>(D, s, Z);
    tend(L, q);
}

void projection_only(const Dev& D, const Launch& L) {
    const int q = tbegin(L, K_PROJECTION);
    k_projection<<<L.nblk_rows, BS_THREADS, 0, L.stream>>>(D);
    tend(L, q);
}

void cell_max_timestep(const Dev& D, const Launch& L, int do_cellmax, int do_timestep) {
    if (do_cellmax) {
        const int q = tbegin(L, K_CELLMAX);
        k_cellmax<<<gdiv(D.ncell_total, BS_THREADS), BS_THREADS, 0, L.stream>>>(D, 1);
        tend(L, q);
    }
    if (do_timestep) {
        int q = tbegin(L, K_TIMESTEP);
        k_scene_max<<<gdiv(D.ncell_total, BS_THREADS), BS_THREADS, 0, L.stream>>>(D);
        tend(L, q);
        q = tbegin(L, K_TIMESTEP);
        k_timestep<<<gdiv(D.nscene, 64), 64, 0, L.stream>>>(D);
        tend(L, q);
    }
}

void advance_time(const Dev& D, const Launch& L) {
    const int q = tbegin(L, K_ADVANCE);
    k_advance_time<<<gdiv(D.nscene, 64), 64, 0, L.stream>>>(D);
    tend(L, q);
}

void snapshot(const Launch& L, const SnapArgs& a) {
    if (a.n <= 0) return;
    const int q = tbegin(L, K_DERIVE);
    k_snapshot<<<gdiv(a.n, BS_THREADS), BS_THREADS, 0, L.stream>>>(a);
    tend(L, q);
}

void upload_gather(const Dev& D, const Launch& L, int row0, int n, int cell0, int has_flags, int has_pid) {
    if (n <= 0) return;
    const int q = tbegin(L, K_DERIVE);
    k_upload_gather<<<gdiv(n, BS_THREADS), BS_THREADS, 0, L.stream>>>(D, row0, n, cell0, has_flags, has_pid);
    tend(L, q);
}

void derive_fields(const Dev& D, const Launch& L) {
    const int q = tbegin(L, K_DERIVE);
    k_derive<<<L.nblk_rows, BS_THREADS, 0, L.stream>>>(D);
    tend(L, q);
}

const char* const kernel_names[K_COUNT] = {
    "rank", "cell_prefix", "scan_cells", "permute", "search_effpor", "freesurf", "eddy", "int_vel",
    "assemble", "comp_vel_pos", "cell_max", "timestep", "shift", "apply_density", "disp", "scalar",
    "bicg_init", "bicg_it1_spmv", "bicg_it2_spmv", "bicg_it3_axpy", "true_residual", "advance_time",
    "derive", "velmag", "projection", "mx_init", "mx_it1_spmv", "mx_it2_spmv", "mx_it3_axpy",
    "mx_residual", "mx_convert", "bicg_p_update", "bicg_s_update", "mx_update", "mg_galerkin0",
    "mg_galerkin", "mg_l0_down", "mg_down", "mg_coarse", "mg_up", "mg_l0_up", "mg_l0_prolong",
    "mg_resid", "relpos", "wc_continuity", "wc_rows", "wc_wall_pressure",
    "fg_start", "fg_put", "fg_arnoldi_spmv", "fg_project", "fg_update", "buffer_exchange", "wall_ghost", "mg_subtree", "collision_shift", "mg_l0_restrict", "mg_tail"};

// Accumulate the finished launches of the ring in order; with wait, block on
// the oldest pending end event (used when the ring is full).
void timer_collect(KTimer* T, bool wait) {
    if (!T || !T->ready) return;
    while (T->tail < T->head) {
        const int q = (int)(T->tail % (KTimer::NEV / 2));
        if (wait) cudaEventSynchronize(T->ev[2 * q + 1]);
        else if (cudaEventQuery(T->ev[2 * q + 1]) != cudaSuccess) break;
        float ms = 0.f;
        if (cudaEventElapsedTime(&ms, T->ev[2 * q], T->ev[2 * q + 1]) == cudaSuccess) {
            T->total_ms[T->id_of[q]] += ms;
            T->count[T->id_of[q]] += 1;
        }
        ++T->tail;
        wait = false;
    }
}

}  // namespace bs
