// bs_sweep.cu -- neighbour search and the neighbour-list sweeps of one ISPH
// step.  One thread per particle row; the neighbour list of a 32-row slice
// is read column by column (sliced ELL), so every warp-wide read of the k-th
// neighbour entry is one coalesced request.  Template parameter T is the
// storage/arithmetic type of the per-pair data (dist, 1/(r^2+lam), grad W)
// and of the sweep sums: double for the FP64 drop-in, float for the mixed
// form.  Positions and the exact pair test are always FP64.
#include "bs_internal.cuh"

namespace {

struct RowCtx {
    int r, s;
    bool active;   // a particle row of a scene that is not held
    bool held;     // a particle row of a held scene
};

__device__ __forceinline__ RowCtx row_ctx(const Dev& D) {
    RowCtx c;
    c.r = blockIdx.x * blockDim.x + threadIdx.x;
    c.s = D.blk_scene[c.r / BS_ALIGN];   // the block's scene, whatever the block size
    const bool row = c.r < D.par[c.s].row0 + D.dyn[c.s].n;
    c.held = row && D.dyn[c.s].hold;
    c.active = row && !c.held;
    return c;
}

// The four cells of the quadrant stencil in the reference's order
// (search.f90:328-388): cell q lies (di0 + (q & 1), dj0 + (q >> 1)) rows and
// columns from the row's cell c, i.e. at c + dj celly + di.  ordp packs
// effpor's order of the same four (porous.f90:125-176: the row's own cell,
// then the other three of the quadrant as listed), two bits per entry.
// False for a non-finite position.
__device__ __forceinline__ bool quad_cells(const ScenePar& P, int c, double xi, double yi, int& di0, int& dj0,
                                          int& ordp) {
    const int lc = c - P.cell0;
    const int i = lc % P.celly + 1, j = lc / P.celly + 1;
    const double xl = cell_xleft(P, j), xr = cell_xright(P, j);
    const double yb = cell_ybot(P, i), yt = cell_ytop(P, i);
    const double mx = xl + fabs((xl - xr) / 2.0);
    const double my = yb + fabs((yt - yb) / 2.0);
    if (xi <= mx && yi <= my) {
        di0 = 0; dj0 = -1; ordp = 2 | 0 << 2 | 3 << 4 | 1 << 6;
    } else if (xi > mx && yi <= my) {
        di0 = 0; dj0 = 0; ordp = 0 | 2 << 2 | 1 << 4 | 3 << 6;
    } else if (xi > mx && yi > my) {
        di0 = -1; dj0 = 0; ordp = 1 | 2 << 2 | 0 << 4 | 3 << 6;
    } else if (xi <= mx && yi > my) {
        di0 = -1; dj0 = -1; ordp = 3 | 2 << 2 | 0 << 4 | 1 << 6;
    } else {
        return false;
    }
    return true;
}

// Corner of the cell (dj, di) steps away relative to the row's own cell
// corner, in FP32: cell_xleft advances by the cell width 4h per column and
// cell_ybot falls by 4h per row (setup.f90:120-123).
__device__ __forceinline__ void cell_offset(float cwf, int dj, int di, float& ox, float& oy) {
    ox = (float)dj * cwf;
    oy = (float)(-di) * cwf;
}

// FP32 position of every row relative to its cell's corner (the search's
// candidate prefilter reads 8 bytes per candidate and no FP64) and, in the
// mixed form, the double-float position the pair offsets are taken from
__global__ void k_relpos(Dev D) {
    const RowCtx R = row_ctx(D);
    if (!R.active) return;
    const ScenePar& P = D.par[R.s];
    const int r = R.r;
    const int lc = D.cell[r] - P.cell0;
    const int i = lc % P.celly + 1, j = lc / P.celly + 1;
    const double x = D.x[r], y = D.y[r];
    D.xr[r] = (float)(x - cell_xleft(P, j));
    D.yr[r] = (float)(y - cell_ybot(P, i));
    if (P.precision == BS_PREC_MIXED) {
        D.pos4[r] = f2_split2(x, y);
        D.volf2[r] = f2_split(D.vol[r]);
    }
}

template <typename T>
__device__ __forceinline__ T ld(const void* p, long e) { return ((const T*)p)[e]; }
template <typename T>
__device__ __forceinline__ void st(void* p, long e, T v) { ((T*)p)[e] = v; }

// ------------------------------------------------------------------ search
// nsearch2 (search.f90:13-308) and effpor/porsearch (porous.f90:32-224)
template <typename T>
__global__ void __launch_bounds__(BS_THREADS) k_search(Dev D, int do_search, int do_effpor) {
    const RowCtx R = row_ctx(D);
    if (!R.active) {
        if (R.held && do_effpor) {   // keep a held scene's density across the buffer swap
            D.rho_new[R.r] = D.rho[R.r];
            D.vol_new[R.r] = D.vol[R.r];
        }
        return;
    }
    const ScenePar& P = D.par[R.s];
    const int r = R.r;
    const int tid = D.tid[r];
    const double xi = D.x[r], yi = D.y[r];
    const int c = D.cell[r];
    int di0, dj0, ordp;
    const bool ok = quad_cells(P, c, xi, yi, di0, dj0, ordp);
    const float cwf = (float)P.cw;
    uint8_t fl = D.flags[r];
    if (do_search) {
        const int kmax = D.kmax;
        const double twoh = P.twoh;
        // Phase 1 (divergent candidate scan): FP32 prefilter of the squared
        // distance from positions relative to the cell corners (rounding
        // error of d^2 below 2e-6 relative for coordinates within a cell) --
        // outside [lo, hi] the exact FP64 test cannot disagree -- and the
        // exact test of functions.f90:38 / search.f90:59 (IEEE sqrt, no FMA,
        // FP64 positions) inside it.  Only indices are appended, so the
        // warp's divergence is cheap.
        const float t2f = (float)(twoh * twoh);
        const float thr_hi = t2f * (1.0f + 1e-5f), thr_lo = t2f * (1.0f - 1e-5f);
        int cnt = 0;
        auto test = [&](int rj, float fx, float fy) {
            const float d2f = fx * fx + fy * fy;
            if (d2f > thr_hi) return;
            if (d2f >= thr_lo) {
                const double dx = __ldg(D.x + rj) - xi, dy = __ldg(D.y + rj) - yi;
                const double rad = __dsqrt_rn(__dadd_rn(__dmul_rn(dx, dx), __dmul_rn(dy, dy)));
                if (!(rad < twoh)) return;
            }
            if (cnt < kmax) D.nidx[ell(r, cnt, kmax)] = rj;
            ++cnt;
        };
        if (ok) {
            const float xri = D.xr[r], yri = D.yr[r];
            for (int q = 0; q < 4; ++q) {
                const int di = di0 + (q & 1), dj = dj0 + (q >> 1);
                const int cq = c + dj * P.celly + di;
                float ox, oy;
                cell_offset(cwf, dj, di, ox, oy);
                const int r1 = D.cell_end[cq];
                int rj = D.cell_start[cq];
                for (; rj + 1 < r1; rj += 2) {   // two independent candidate loads in flight
                    const float x0 = __ldg(D.xr + rj) + ox, y0 = __ldg(D.yr + rj) + oy;
                    const float x1 = __ldg(D.xr + rj + 1) + ox, y1 = __ldg(D.yr + rj + 1) + oy;
                    if (rj != r) test(rj, x0 - xri, y0 - yri);   // (tid, matid) self-exclusion
                    if (rj + 1 != r) test(rj + 1, x1 - xri, y1 - yri);
                }
                if (rj < r1 && rj != r) test(rj, (__ldg(D.xr + rj) + ox) - xri, (__ldg(D.yr + rj) + oy) - yri);
            }
        }
        if (cnt > kmax) set_err(D, R.s, BS_ERR_NBR_OVERFLOW);
        const int n = cnt < kmax ? cnt : kmax;
        D.ncount[r] = n;
        // Phase 2 (uniform over the accepted neighbours): pair quantities and
        // the gradient-correction sums (search.f90:61-85).
        double a00 = 0.0, a01 = 0.0, a10 = 0.0, a11 = 0.0;
        if (sizeof(T) == 4) {
            // mixed: the pair quantities are stored in FP32 and computed on
            // the FP32 pipe from double-float positions: the offset x_j - x_i
            // (f2_diff, ~1e-13 m), r, r^2 and 1/r (pair_r, ~2^-44 before
            // rounding) and 1/(r^2 + lam) by a double-float Newton step, each
            // the FP32 rounding of the FP64 value up to ties.  The kernel
            // gradient is F = S g(q),
            // q = r/h, with one FP32 scale S = cn1/h^2:
            //   q < 1: g = (9q - 12) + (cn2/cn1)(3q - 6/q)
            //   q >= 1: g = -3 (1 + cn2/cn1) (2 - q)^2 / q
            // g in double-float arithmetic (q, 1/q and the ratios as (hi, lo)
            // pairs) and each stored component F (x_i - x_j) rounded once.
            // Wall particles sit on a lattice and fluid particles stay near
            // one, so many pairs share an offset and the same rounding: FP32
            // arithmetic in F would act as a small change of the kernel's
            // shape, which no sum averages out (~1e-6 in the pressure of
            // coarse scenes); so would FP32 constants per term (1/h, 1/h^2,
            // 1/h^3, cn1, cn2 each rounded).  S is the same for every
            // gradient of the scene: it cancels in the corrected gradients
            // and the Jacobi-scaled rows and elsewhere acts as one rounded
            // constant.  The correction sums take the components before their
            // rounding times V (x_j - x_i), all as (hi, lo) pairs, into
            // double-float accumulators, as the FP64 form sums its unrounded
            // values: the correction matrix multiplies every pair of the row,
            // so its errors do not average out either.
            float2 s00 = make_float2(0.f, 0.f), s01 = s00, s10 = s00, s11 = s00;
            const float kqs = P.kq_s;
            const float2 kr = make_float2(P.kq_rho_h, P.kq_rho_l), k3 = make_float2(P.kq_k3_h, P.kq_k3_l);
            const float2 hf = f2_split(P.h), ihd = f2_split(P.inv_h);
            const float2 lam = make_float2(P.kq_lam_h, P.kq_lam_l);
            const float4 pi4 = D.pos4[r];
            for (int k = 0; k < n; ++k) {
                const long e = ell(r, k, kmax);
                const int rj = D.nidx[e];
                const float4 pj4 = __ldg(D.pos4 + rj);
                const float2 dx = f2_diff(pj4.x, pj4.y, pi4.x, pi4.y);
                const float2 dy = f2_diff(pj4.z, pj4.w, pi4.z, pi4.w);
                const PairR pr = pair_r(dx, dy);
                const float rad = pr.rh;
                const float rinv = f2_rcp(f2_add(make_float2(pr.sh, pr.sl), lam)).x;
                const float2 q = f2_mul(make_float2(pr.rh, pr.rl), ihd);
                const float2 iq = f2_rcp(q);
                float2 g;
                if (f2_less(pr.rh, pr.rl, hf.x, hf.y)) {
                    const float2 t1 = f2_add(f2_mulf(q, 9.0f), make_float2(-12.0f, 0.0f));
                    const float2 t2 = f2_add(f2_mulf(q, 3.0f), f2_mulf(iq, -6.0f));
                    g = f2_add(t1, f2_mul(kr, t2));
                } else {
                    const float2 s = f2_two_sum(2.0f, -q.x);
                    const float2 a = f2_fast_two_sum(s.x, __fsub_rn(s.y, q.y));
                    g = f2_mul(k3, f2_mul(f2_mul(a, a), iq));
                    g = make_float2(-g.x, -g.y);
                }
                const float2 F = f2_mulf(g, kqs);
                // F (x_i - x_j) as (hi, lo); hi is the stored FP32 value
                float2 kx2 = f2_mul(F, dx), ky2 = f2_mul(F, dy);
                kx2 = make_float2(-kx2.x, -kx2.y);
                ky2 = make_float2(-ky2.x, -ky2.y);
                const float kx = kx2.x, ky = ky2.x;
                st<T>(D.ndist, e, (T)rad);
                st<T>(D.nrinv, e, (T)rinv);
                st<T>(D.nkx, e, (T)kx);
                st<T>(D.nky, e, (T)ky);
                // V (dx hi + dx lo) as (hi, lo) from V as (hi, lo)
                const float2 vj = __ldg(D.volf2 + rj);
                const float r1h = __fmul_rn(vj.x, dx.x);
                const float r1e = __fmaf_rn(vj.y, dx.x, __fmaf_rn(vj.x, dx.y, __fmaf_rn(vj.x, dx.x, -r1h)));
                const float r3h = __fmul_rn(vj.x, dy.x);
                const float r3e = __fmaf_rn(vj.y, dy.x, __fmaf_rn(vj.x, dy.y, __fmaf_rn(vj.x, dy.x, -r3h)));
                f2_acc_prod(s00, kx2, r1h, r1e);
                f2_acc_prod(s01, ky2, r1h, r1e);
                f2_acc_prod(s10, kx2, r3h, r3e);
                f2_acc_prod(s11, ky2, r3h, r3e);
            }
            a00 = (double)s00.x + (double)s00.y;
            a01 = (double)s01.x + (double)s01.y;
            a10 = (double)s10.x + (double)s10.y;
            a11 = (double)s11.x + (double)s11.y;
        }
        for (int k = 0; k < (sizeof(T) == 4 ? 0 : n); ++k) {
            const long e = ell(r, k, kmax);
            const int rj = D.nidx[e];
            const double dx = __ldg(D.x + rj) - xi, dy = __ldg(D.y + rj) - yi;
            const double rad = __dsqrt_rn(__dadd_rn(__dmul_rn(dx, dx), __dmul_rn(dy, dy)));
            const double ir = 1.0 / rad;
            const double rinv = 1.0 / (rad * rad + P.lam);
            double F;
            if (rad < P.h) {
                F = P.cn1 * (9.0 * rad * P.inv_h3 - 12.0 * P.inv_h2) + P.cn2 * (3.0 * rad * P.inv_h3 - 6.0 * P.inv_h * ir);
            } else {
                const double a = 2.0 - rad * P.inv_h;
                F = -(P.cn1 + P.cn2) * (3.0 * P.inv_h * ir) * a * a;
            }
            const double kx = F * (-dx), ky = F * (-dy);   // grad_i W = F (r_i - r_j)
            st<T>(D.ndist, e, (T)rad);
            st<T>(D.nrinv, e, (T)rinv);
            st<T>(D.nkx, e, (T)kx);
            st<T>(D.nky, e, (T)ky);
            const double vj = D.vol[rj];
            const double res1 = vj * dx, res3 = vj * dy;
            a00 += kx * res1;
            a01 += ky * res1;
            a10 += kx * res3;
            a11 += ky * res3;
        }
        fl &= ~BS_FLAG_FREE;
        double gv = 0.0;
        if (tid == BS_TID_FLUID) {
            fl &= ~BS_FLAG_VICINITY;
            gv = a00 + a11;
            // invertmat2D, functions.f90:62-96
            const double det = a00 * a11 - a01 * a10;
            double c0 = 1.0, c1 = 0.0, c2 = 0.0, c3 = 1.0;
            if (fabs(det) >= BS_SP1EM5 && isfinite(det)) {
                // mixed: 1/det by a Newton step from the FP32 reciprocal
                // (~1e-14; det is a sum of FP32-accurate terms)
                const double id = sizeof(T) == 4 ? fast_rcp64(det) : 1.0 / det;
                c0 = a11 * id;
                c1 = -a01 * id;
                c2 = -a10 * id;
                c3 = a00 * id;
            }
            D.c0[r] = c0; D.c1[r] = c1; D.c2[r] = c2; D.c3[r] = c3;
            if (sizeof(T) == 4) {
                const float2 a = f2_split(c0), b = f2_split(c1), cc = f2_split(c2), d = f2_split(c3);
                D.cfa[r] = make_float4(a.x, a.y, b.x, b.y);
                D.cfb[r] = make_float4(cc.x, cc.y, d.x, d.y);
            }
            if ((gv <= P.freethr) && !(fl & BS_FLAG_BUFFER)) fl |= BS_FLAG_FREE;
        }
        D.gradvx[r] = gv;
        D.flags[r] = fl;
    }
    if (do_effpor) {
        double phi = 1.0, res = 0.0;
        if (tid == BS_TID_FLUID) {
            double sf = 0.0;
            if (ok) {
                // effpor's cell order (porous.f90:125-176): its own cell, then
                // the other three of the same quadrant in the listed order
                const double wsolid = 1.0 - P.por * 1.0;
                const float wsf = (float)wsolid, t2c = (float)(P.twoh * P.twoh);
                Kahan32 sff;
                const KerF KF = ker_f(P);
                const float t2f = (float)(P.twoh * P.twoh) * (1.0f + 1e-5f);
                const float xri = D.xr[r], yri = D.yr[r];
                float4 pi4 = make_float4(0.f, 0.f, 0.f, 0.f);
                if (sizeof(T) == 4) pi4 = D.pos4[r];
                for (int k = 0; k < 4; ++k) {
                    const int q = (ordp >> (2 * k)) & 3;
                    const int di = di0 + (q & 1), dj = dj0 + (q >> 1);
                    const int cq = c + dj * P.celly + di;
                    float ox, oy;
                    cell_offset(cwf, dj, di, ox, oy);
                    const int g1 = D.gcell_end[cq];
                    for (int g = D.gcell_start[cq]; g < g1; ++g) {
                        // FP32 prefilter (as in the neighbour scan): a grain
                        // rejected here is outside 2h in FP64 as well
                        const float fx = (__ldg(D.gxr + g) + ox) - xri, fy = (__ldg(D.gyr + g) + oy) - yri;
                        if (fx * fx + fy * fy > t2f) continue;
                        if (sizeof(T) == 4) {
                            // mixed: FP32 (W(2h) = 0: the cut needs no exact
                            // test), the offset from the double-float positions
                            const float4 g4 = __ldg(D.gpos4 + g);
                            const float ex = f2_diff(pi4.x, pi4.y, g4.x, g4.y).x;
                            const float ey = f2_diff(pi4.z, pi4.w, g4.z, g4.w).x;
                            const float s2 = ex * ex + ey * ey;
                            if (s2 < t2c) {
                                float rad = 0.0f;   // grains may coincide with pore particles
                                if (s2 > 0.0f) {
                                    float ir = rsqrtf(s2);
                                    ir = ir * (1.5f - 0.5f * s2 * ir * ir);
                                    rad = s2 * ir;
                                }
                                sff.add(wsf * bs_Wf(rad, KF) * (float)D.gv[g]);
                            }
                        } else {
                            const double dx = xi - D.gx[g], dy = yi - D.gy[g];
                            const double rad = __dsqrt_rn(__dadd_rn(__dmul_rn(dx, dx), __dmul_rn(dy, dy)));
                            if (rad < P.twoh) sf = sf + wsolid * bs_W(rad, P) * D.gv[g];
                        }
                    }
                }
                if (sizeof(T) == 4) sf = sff.value();
            }
            if (sf > (1.0 - P.por)) sf = 1.0 - P.por;
            phi = 1.0 - sf;
            const double od = D.oden[r];
            const double rn = phi * od;
            if (do_effpor == 2) {   // WCSPH: the density is the continuity equation's
                D.rho_new[r] = D.rho[r];
                D.vol_new[r] = D.vol[r];
            } else {
                D.rho_new[r] = rn;
                D.vol_new[r] = sizeof(T) == 4 ? D.mass[r] * fast_rcp64(rn) : D.mass[r] / rn;
            }
            const double phi3 = phi * phi * phi;
            const double vx = D.vx[r], vy = D.vy[r];
            if (sizeof(T) == 4) {
                // mixed: the same drag with Newton-step reciprocals and square
                // roots (~1e-13 relative) in place of IEEE division and sqrt
                double sp3, isp3, vm = 0.0, slk = 0.0, t;
                fast_r64(150.0 * phi3, t, isp3);
                const double Fch = 1.750 * isp3;
                fast_r64(phi3, sp3, t);
                const double v2 = vx * vx + vy * vy;
                if (v2 > 0.0) fast_r64(v2, vm, t);
                if (P.lamk > 0.0) fast_r64(P.lamk, slk, t);
                const double om = 1.0 - phi;
                res = -(bs_vis(od) * fast_rcp64(od) * P.lamk * (om * om) * fast_rcp64(phi3 * (P.d50 * P.d50))) -
                      (Fch * vm * slk * om * fast_rcp64(sp3 * P.d50));
            } else {
                const double Fch = 1.750 / sqrt(150.0 * phi3);
                const double vm = sqrt(vx * vx + vy * vy);
                res = -((bs_vis(od) / od) * P.lamk * ((1.0 - phi) * (1.0 - phi)) / (phi3 * (P.d50 * P.d50))) -
                      ((Fch * vm * sqrt(P.lamk) * (1.0 - phi)) / (sqrt(phi3) * P.d50));
            }
        } else {
            D.rho_new[r] = D.rho[r];
            D.vol_new[r] = D.vol[r];
        }
        D.por[r] = phi;
        D.resx[r] = res;
        D.resy[r] = res;
    }
}

// freesurf, isph.f90:49-86 (concurrent writes of the same bit: benign)
__global__ void k_freesurf(Dev D) {
    const RowCtx R = row_ctx(D);
    if (!R.active) return;
    const int r = R.r;
    const uint8_t fl = D.flags[r];
    if (D.tid[r] != BS_TID_FLUID || (fl & BS_FLAG_BUFFER)) return;
    if (!(D.gradvx[r] <= D.par[R.s].freethr)) return;
    const int n = D.ncount[r];
    for (int k = 0; k < n; ++k) {
        const int j = D.nidx[ell(r, k, D.kmax)];
        D.flags[j] = D.flags[j] | BS_FLAG_VICINITY;
    }
}

// ------------------------------------------------------------------ eddyvis
// turbulence.f90:12-113, with int_vel's varts (integrator.f90:468-507: the
// same L-corrected velocity-gradient sums) and optionally the per-particle
// dispersion tensor used by the next scalar sub-steps (scalar.f90:276-301).
template <typename T>
__global__ void __launch_bounds__(BS_THREADS) k_eddy(Dev D, int with_eddy, int with_varts, int with_disp) {
    const RowCtx R = row_ctx(D);
    if (!R.active) return;
    const ScenePar& P = D.par[R.s];
    const int r = R.r;
    if (D.tid[r] != BS_TID_FLUID) {
        if (with_eddy) {
            D.nut[r] = 0.0;
            D.tke[r] = 0.0;
        }
        if (with_varts) D.varts[r] = 0.0;
        return;
    }
    const T c0 = (T)D.c0[r], c1 = (T)D.c1[r], c2 = (T)D.c2[r], c3 = (T)D.c3[r];
    const double phi = D.por[r];
    const double vx = D.vx[r], vy = D.vy[r];
    const T ui = (T)D.qu[r], wi = (T)D.qw[r];   // vx/phi, vy/phi (k_quot)
    T t1 = 0, t2 = 0, t3 = 0;
    const int n = D.ncount[r];
    const int kmax = D.kmax;
    if (sizeof(T) == 4) {
        // mixed: the neighbours' u/phi, w/phi as (hi, lo) pairs and volumes
        // from the k_quot records, the differences rounded once to FP32
        const float4 q4 = D.rec0[r];
        const CorrF cf = corr_f(D, r);
        for (int k = 0; k < n; ++k) {
            const long e = ell(r, k, kmax);
            const int j = D.nidx[e];
            const float z1 = ld<float>(D.nkx, e), z2 = ld<float>(D.nky, e);
            const float4 qj = __ldg(D.rec0 + j);
            const float a = f2_diff(qj.x, qj.y, q4.x, q4.y).x, b = f2_diff(qj.z, qj.w, q4.z, q4.w).x;
            const float V = __ldg(D.rec1 + j).x;
            const float Lx = cf.lx(z1, z2), Ly = cf.ly(z1, z2);
            t1 += V * a * Lx;
            t2 += V * b * Ly;
            t3 += 0.5f * V * (a * Ly + b * Lx);
        }
    }
    for (int k = 0; k < (sizeof(T) == 4 ? 0 : n); ++k) {
        const long e = ell(r, k, kmax);
        const int j = D.nidx[e];
        const T z1 = ld<T>(D.nkx, e), z2 = ld<T>(D.nky, e);
        const T a = (T)D.qu[j] - ui, b = (T)D.qw[j] - wi;
        const T V = (T)D.vol[j];
        const T Lx = c0 * z1 + c1 * z2, Ly = c2 * z1 + c3 * z2;
        t1 += V * a * Lx;
        t2 += V * b * Ly;
        t3 += (T)0.5 * V * (a * Ly + b * Lx);
    }
    const double cs = 0.150, cv = 0.080, ce = 1.0, dl = P.dl;
    const double t4 = sqrt(2.0 * ((double)t1 * t1 + (double)t2 * t2) + (2.0 * t3) * (2.0 * t3));
    double nut = D.nut[r];
    if (with_eddy) {
        nut = ((cs * dl) * (cs * dl)) * t4;
        D.nut[r] = nut;
        D.tke[r] = (cv / ce) * ((dl * t4) * (dl * t4));
    }
    if (with_varts) {
        double va = 0.0;
        if (D.flags[r] & BS_FLAG_FREE)
            va = (dl * dl) * sqrt((double)t1 * t1 + (double)t2 * t2) * sqrt(vx * vx + vy * vy) /
                 ((D.dyn[R.s].umax + BS_SP1EM6) * phi);
        D.varts[r] = va;
    }
    if (with_disp) {
        const double al = 0.0025, at = 0.00025, Dm = BS_SP1EM9;
        const double vi = sqrt(vx * vx + vy * vy) / phi;
        const double dl_ = sqrt((al * vi) + Dm) * vi * phi, dt_ = sqrt((at * vi) + Dm) * vi * phi;
        D.Dp0[r] = vx / dl_;
        D.Dp1[r] = vy / dl_;
        D.Dp2[r] = (-vy) / dt_;
        D.Dp3[r] = vx / dt_;
        D.Dt[r] = Dm + nut / P.tschmidt;
    }
}

// ------------------------------------------------------------------ int_vel
// integrator.f90:510-701 (non-pressure velocity v*)
template <typename T>
__global__ void __launch_bounds__(BS_THREADS) k_intvel(Dev D) {
    const RowCtx R = row_ctx(D);
    if (!R.active) return;
    const ScenePar& P = D.par[R.s];
    const int r = R.r;
    if (D.tid[r] != BS_TID_FLUID) return;
    const uint8_t fl = D.flags[r];
    const double dt = D.dyn[R.s].dt;
    const double phi = D.por[r];
    if (fl & BS_FLAG_BUFFER) {
        D.vxs[r] = D.vx[r];
        D.vys[r] = P.g * phi * dt;
        return;
    }
    const T c0 = (T)D.c0[r], c1 = (T)D.c1[r], c2 = (T)D.c2[r], c3 = (T)D.c3[r];
    const double xi = D.x[r], yi = D.y[r], vxi = D.vx[r], vyi = D.vy[r];
    const double nui = D.nu[r], nuti = D.nut[r], tkei = D.tke[r], vartsi = D.varts[r];
    const bool freei = fl & BS_FLAG_FREE;
    T sx = 0, sy = 0;
    const int n = D.ncount[r];
    const int kmax = D.kmax;
    const T two3 = (T)(2.0 / 3);
    double sxd = 0.0, syd = 0.0;   // the sums as the final update reads them
    if (sizeof(T) == 4) {
        // mixed: everything a pair reads of its neighbour from the k_quot
        // records (positions, velocities and tke as (hi, lo) pairs, the
        // viscosities, volume and varts in FP32, nut < 1e-6 as a flag), on
        // the FP32 pipe with compensated sums
        const float4 pi4 = D.pos4[r], vi4 = D.rec0[r], ki4 = D.rec1[r];
        const float nuif = ki4.w, nutif = ki4.z, vartsif = D.rec2[r].y;
        const bool nutis = nuti < BS_SP1EM6;
        const float iwo = (float)(1.0 / P.wo), phif = (float)phi, two3f = (float)(2.0 / 3);
        const KerF KF = ker_f(P);
        const CorrF cf = corr_f(D, r);
        Kahan32 kx, ky;
        for (int k = 0; k < n; ++k) {
            const long e = ell(r, k, kmax);
            const int j = D.nidx[e];
            const float z1 = ld<float>(D.nkx, e), z2 = ld<float>(D.nky, e);
            const float pd = ld<float>(D.nrinv, e);
            const int tj = D.tid[j];
            const float4 kj = __ldg(D.rec1 + j), wj = __ldg(D.rec2 + j);
            float cmu;
            if (tj == BS_TID_FLUID) {   // harmonic mean
                const float nuj = kj.w;
                cmu = 2.0f * nuif * nuj / (nuif + nuj);
            } else {
                cmu = nuif;
            }
            float vart = 0.0f;
            if (freei) vart = vartsif;
            else if (D.flags[j] & BS_FLAG_FREE) vart = bs_Wf(ld<float>(D.ndist, e), KF) * wj.y * iwo;
            const float pvol = wj.x;
            const float Lx = cf.lx(z1, z2), Ly = cf.ly(z1, z2);
            const float4 pj4 = __ldg(D.pos4 + j), vj4 = __ldg(D.rec0 + j);
            const float dxi = f2_diff(pi4.x, pi4.y, pj4.x, pj4.y).x, dyi = f2_diff(pi4.z, pi4.w, pj4.z, pj4.w).x;
            const float gg = 2.0f * pvol * (dxi * Lx + dyi * Ly) * pd;
            const float ax = f2_diff(vi4.x, vi4.y, vj4.x, vj4.y).x * gg;
            const float ay = f2_diff(vi4.z, vi4.w, vj4.z, vj4.w).x * gg;
            kx.add(ax * (cmu + vart));
            ky.add(ay * (cmu + vart));
            if (tj > 2) {
                const float nutj = kj.z;
                float mix;
                if (nutis && wj.z != 0.0f) mix = (nutif + nutj) * 0.5f;
                else mix = (2.0f * nutif * nutj) / (nutif + nutj);
                kx.add(ax * mix);
                ky.add(ay * mix);
            }
            const float tk = pvol * f2_diff(kj.x, kj.y, ki4.x, ki4.y).x;
            kx.add(-(tk * Lx * phif * two3f));
            ky.add(-(tk * Ly * phif * two3f));
        }
        sxd = kx.value();
        syd = ky.value();
    }
    for (int k = 0; k < (sizeof(T) == 4 ? 0 : n); ++k) {
        const long e = ell(r, k, kmax);
        const int j = D.nidx[e];
        const T z1 = ld<T>(D.nkx, e), z2 = ld<T>(D.nky, e);
        const T pd = ld<T>(D.nrinv, e);
        const int tj = D.tid[j];
        T cmu;
        if (tj == BS_TID_FLUID) {   // harmonic mean (FP32 in the mixed form)
            const T nuj = (T)D.nu[j];
            cmu = (T)2 * (T)nui * nuj / ((T)nui + nuj);
        } else {
            cmu = (T)nui;
        }
        T vart = 0;
        if (freei) vart = (T)vartsi;
        else if (D.flags[j] & BS_FLAG_FREE) vart = (T)(bs_W((double)ld<T>(D.ndist, e), P) * D.varts[j] / P.wo);
        const T pvol = (T)D.vol[j];
        const T Lx = c0 * z1 + c1 * z2, Ly = c2 * z1 + c3 * z2;
        const T dxi = (T)(xi - D.x[j]), dyi = (T)(yi - D.y[j]);
        const T gg = (T)2 * pvol * (dxi * Lx + dyi * Ly) * pd;
        const T ax = (T)(vxi - D.vx[j]) * gg, ay = (T)(vyi - D.vy[j]) * gg;
        sx += ax * (cmu + vart);
        sy += ay * (cmu + vart);
        if (tj > 2) {
            const double nutj = D.nut[j];
            T mix;
            if ((nuti < BS_SP1EM6) && (nutj < BS_SP1EM6)) mix = (T)((nuti + nutj) * 0.50);
            else mix = ((T)2 * (T)nuti * (T)nutj) / ((T)nuti + (T)nutj);
            sx += ax * mix;
            sy += ay * mix;
        }
        const T tk = pvol * (T)(D.tke[j] - tkei);
        sx -= tk * Lx * (T)phi * two3;
        sy -= tk * Ly * (T)phi * two3;
    }
    if (sizeof(T) != 4) {
        sxd = (double)sx;
        syd = (double)sy;
    }
    double vxs = (vxi + (dt * sxd)) / (1.0 - dt * D.resx[r] * phi);
    double vys = (vyi + dt * syd) / (1.0 - dt * D.resy[r] * phi);
    vys = vys + P.g * phi * dt;
    D.vxs[r] = vxs;
    D.vys[r] = vys;
}

// ------------------------------------------------------------- assembly
// Per-particle quotients of the neighbour sweeps (FP64 division is the
// costly operation on this part; one division per particle instead of one
// or more per pair) and, in the mixed form, the records the sweep reads of
// a row's neighbours: each field converted to FP32 once per row instead of
// once per pair, a field whose pair differences cancel as a (hi, lo) FP32
// pair (the difference of two pairs rounds to the FP32 rounding of the FP64
// difference), a threshold test on a neighbour's value as a flag taken on
// the FP64 value.  Launched by the sweep's wrapper right before the sweep.
//   mode 0 (assembly): qa = rho/phi, qu = vxs/phi, qw = vys/phi, qi = 1/phi;
//     rec0 = (qu, qw) pairs, rec1 = (vxs, vys) pairs, rec2 = (qa, m/rho, oden, 0)
//   mode 1 (eddyvis): qu = vx/phi, qw = vy/phi; rec0 = (qu, qw) pairs, rec1.x = m/rho
//   mode 2 (comp_vel): qa = rho/phi; rec0 = (p, qa, m/rho, 0)
//   mode 3 (int_vel, mixed only): rec0 = (vx, vy) pairs, rec1 = (tke pair, nut, nu),
//     rec2 = (m/rho, varts, nut < 1e-6, 0)
//   mode 4 (scalar sub-step, mixed only): rec0 = (Dp0, Dp1, Dp2, Dp3),
//     rec1 = (Dt, con, phi, (phi < 0.7) + 2 (nut < 1e-6))
//   mode 5 (opt2_shift, mixed only): rec0 = (vx, vy) pairs, rec1.x = m/rho
//   mode 6 (WCSPH continuity, mixed only): rec0 = (vx, vy) pairs,
//     rec1 = (rho, hydrostatic density) pairs, rec2.x = m
// Modes 0, 3, 4 and 6 also refresh the double-float positions.
__global__ void k_quot(Dev D, int mode) {
    const RowCtx R = row_ctx(D);
    if (!R.active) return;
    const int r = R.r;
    const double phi = D.por[r];
    const bool mixed = D.par[R.s].precision == BS_PREC_MIXED;
    if (mixed && (mode == 0 || mode == 3 || mode == 4 || mode == 6)) D.pos4[r] = f2_split2(D.x[r], D.y[r]);
    switch (mode) {
    case 0: {
        const double ip = 1.0 / phi;
        const double qa = D.rho[r] * ip, qu = D.vxs[r] * ip, qw = D.vys[r] * ip;
        D.qa[r] = qa;
        D.qu[r] = qu;
        D.qw[r] = qw;
        D.qi[r] = ip;
        if (mixed) {
            D.rec0[r] = f2_split2(qu, qw);
            D.rec1[r] = f2_split2(D.vxs[r], D.vys[r]);
            D.rec2[r] = make_float4((float)qa, (float)D.vol[r], (float)D.oden[r], 0.0f);
        }
        break;
    }
    case 1: {
        const double qu = D.vx[r] / phi, qw = D.vy[r] / phi;
        D.qu[r] = qu;
        D.qw[r] = qw;
        if (mixed) {
            D.rec0[r] = f2_split2(qu, qw);
            D.rec1[r] = make_float4((float)D.vol[r], 0.0f, 0.0f, 0.0f);
        }
        break;
    }
    case 2: {
        const double qa = D.rho[r] / phi;
        D.qa[r] = qa;
        if (mixed) D.rec0[r] = make_float4((float)D.p[r], (float)qa, (float)D.vol[r], 0.0f);
        break;
    }
    case 3: {
        const double nut = D.nut[r];
        D.rec0[r] = f2_split2(D.vx[r], D.vy[r]);
        const float2 tk = f2_split(D.tke[r]);
        D.rec1[r] = make_float4(tk.x, tk.y, (float)nut, (float)D.nu[r]);
        D.rec2[r] = make_float4((float)D.vol[r], (float)D.varts[r], nut < BS_SP1EM6 ? 1.0f : 0.0f, 0.0f);
        break;
    }
    case 4: {
        D.rec0[r] = make_float4((float)D.Dp0[r], (float)D.Dp1[r], (float)D.Dp2[r], (float)D.Dp3[r]);
        const float bits = (phi < 0.7 ? 1.0f : 0.0f) + (D.nut[r] < BS_SP1EM6 ? 2.0f : 0.0f);
        D.rec1[r] = make_float4((float)D.Dt[r], (float)D.con[r], (float)phi, bits);
        break;
    }
    case 5: {
        D.rec0[r] = f2_split2(D.vx[r], D.vy[r]);
        D.rec1[r] = make_float4((float)D.vol[r], 0.0f, 0.0f, 0.0f);
        break;
    }
    case 6: {
        D.rec0[r] = f2_split2(D.vx[r], D.vy[r]);
        D.rec1[r] = f2_split2(D.rho[r], D.whyd[r]);
        D.rec2[r] = make_float4((float)D.mass[r], 0.0f, 0.0f, 0.0f);
        break;
    }
    }
}

// The mixed form of the assembly: the same entries and right-hand side on
// the FP32 pipe.  Pair offsets and the cancelling differences (u/phi, w/phi,
// vxs, vys of the pair) are taken from double-float copies (pos4 and the
// k_quot records), the matrix entries in FP32 with a compensated diagonal.
// The right-hand side is a divergence: its pair terms cancel to a small sum,
// which would carry each term's FP32 rounding many times over, so each term
// (the velocity difference and the corrected gradient as (hi, lo) pairs, their
// dot product) is double-float and so is the sum; the density and volume
// factors, smooth over a row's pairs, stay FP32.  The Jacobi scaling writes
// the FP64 values and their double-float split (aval32 + aval_lo) for the
// solver.
__device__ __forceinline__ void assemble_mixed(const Dev& D, const RowCtx& R) {
    const ScenePar& P = D.par[R.s];
    const int r = R.r;
    const int ti = D.tid[r];
    const uint8_t fl = D.flags[r];
    const float4 pi4 = D.pos4[r];
    const float4 ui = D.rec0[r], vi = D.rec1[r];
    const float ai = D.rec2[r].x;                       // rho_i/phi_i
    const float bi = (float)(D.qa[r] * D.qi[r]);          // rho_i/phi_i^2
    const CorrF cf = corr_f(D, r);
    const bool freei = fl & BS_FLAG_FREE;
    const float lampf = (float)(1.0 / (P.rho * P.rel_den));
    const float voli = ti == BS_TID_WALL ? (float)(D.mass[r] / D.rho[r]) : 0.0f;
    const int n = D.ncount[r];
    const int kmax = D.kmax;
    float* a32 = D.aval32;
    Kahan32 dia;
    float2 fv = make_float2(0.0f, 0.0f);
    for (int k = 0; k < n; ++k) {
        const long e = ell(r, k, kmax);
        const int j = D.nidx[e];
        const float z1 = ld<float>(D.nkx, e), z2 = ld<float>(D.nky, e);
        const float pd = ld<float>(D.nrinv, e);
        const int tj = D.tid[j];
        const float4 pj4 = __ldg(D.pos4 + j);
        const float dxi = f2_diff(pi4.x, pi4.y, pj4.x, pj4.y).x;   // x_i - x_j
        const float dyi = f2_diff(pi4.z, pi4.w, pj4.z, pj4.w).x;
        float off = 0.0f;
        if (ti == BS_TID_FLUID) {
            const float4 aj4 = __ldg(D.rec2 + j);
            const float lamp = (freei && tj == BS_TID_FLUID) ? (1.0f + aj4.z * lampf) : 1.0f;
            const float pvol = aj4.y;
            const float2 Lx = cf.lx2(z1, z2), Ly = cf.ly2(z1, z2);
            const float t12 = 2.0f * pvol * (Lx.x * dxi + Ly.x * dyi) * pd;
            off = -t12;
            dia.add(t12 * lamp);
            float2 ax, ay;
            if (tj == BS_TID_FLUID) {
                const float aj = aj4.x;
                const float rho_ij = 2.0f * aj * ai / (aj + ai);
                const float4 uj = __ldg(D.rec0 + j);
                ax = f2_mulf(f2_diff(uj.x, uj.y, ui.x, ui.y), rho_ij);
                ay = f2_mulf(f2_diff(uj.z, uj.w, ui.z, ui.w), rho_ij);
            } else {
                const float4 vj = __ldg(D.rec1 + j);
                ax = f2_mulf(f2_diff(vj.x, vj.y, vi.x, vi.y), bi);
                ay = f2_mulf(f2_diff(vj.z, vj.w, vi.z, vi.w), bi);
            }
            fv = f2_add(fv, f2_mulf(f2_add(f2_mul(ax, Lx), f2_mul(ay, Ly)), pvol));
        } else if (ti == BS_TID_GHOST) {
            if (tj <= 2) {
                const float t12 = 2.0f * __ldg(D.rec2 + j).y * (z1 * dxi + z2 * dyi) * pd;
                off = -t12;
                dia.add(t12);
            }
        } else if (ti == BS_TID_WALL) {
            if (tj == BS_TID_FLUID) {
                const CorrF cj = corr_f(D, j);
                const float2 Lx = cj.lx2(z1, z2), Ly = cj.ly2(z1, z2);
                const float t12 = 2.0f * voli * (Lx.x * dxi + Ly.x * dyi) * pd;
                off = -t12;
                dia.add(t12);
                // a_j (u_j/phi_j - vxs_i/phi_i): vxs_i/phi_i is the row's own u/phi
                const float aj = __ldg(D.rec2 + j).x;
                const float4 uj = __ldg(D.rec0 + j);
                const float2 ax = f2_mulf(f2_diff(uj.x, uj.y, ui.x, ui.y), aj);
                const float2 ay = f2_mulf(f2_diff(uj.z, uj.w, ui.z, ui.w), aj);
                fv = f2_add(fv, f2_mulf(f2_add(f2_mul(ax, Lx), f2_mul(ay, Ly)), voli));
            } else {
                const float t12 = 2.0f * __ldg(D.rec2 + j).y * (z1 * dxi + z2 * dyi) * pd;
                off = -t12;
                dia.add(t12);
            }
        }
        a32[e] = off;   // unscaled, scaled below
    }
    double extra = 0.0;
    if (ti == BS_TID_GHOST && n > 0) {
        const int j0 = D.nidx[ell(r, 0, kmax)];
        if (j0 < r && D.tid[j0] == BS_TID_FLUID) extra = 1.0;
    }
    const double dd = dia.value();
    if (!(dd != 0.0) || !isfinite(dd)) set_err(D, R.s, BS_ERR_ZERO_DIAG);
    const double inv = fast_rcp64(dd);
    D.adiag[r] = dd / dd + extra * inv;
    D.rhs[r] = ((double)fv.x + (double)fv.y) * fast_rcp64(D.dyn[R.s].dt) * inv;
    // Jacobi scaling: FP64 values for the FP64 residuals, and the
    // double-float split off * (inv hi + inv lo) for the solver's SpMV
    const float2 invd = f2_split(inv);
    double* a = (double*)D.aval;
    for (int k = 0; k < n; ++k) {
        const long e = ell(r, k, kmax);
        const float o = a32[e];
        const float ph = __fmul_rn(o, invd.x);
        const float2 v = f2_fast_two_sum(ph, __fmaf_rn(o, invd.y, __fmaf_rn(o, invd.x, -ph)));
        a32[e] = v.x;
        D.aval_lo[e] = v.y;
        a[e] = (double)o * inv;
    }
    if (r == P.row0) D.dyn[R.s].asm_split = 1;
}

// ppesolve assembly (isph.f90:115-456) with the quotients of k_quot:
// rho_ij = 2 a_j a_i / (a_j + a_i) with a = rho/phi, the velocity terms as
// rho_ij (vxs_j/phi_j - vxs_i/phi_i) -- the reference's expressions
// regrouped, one division per fluid pair
template <typename T>
__global__ void __launch_bounds__(BS_THREADS) k_assemble(Dev D) {
    const RowCtx R = row_ctx(D);
    if (!R.active) return;
    if (sizeof(T) == 4) {
        assemble_mixed(D, R);
        return;
    }
    const ScenePar& P = D.par[R.s];
    const int r = R.r;
    const int ti = D.tid[r];
    const uint8_t fl = D.flags[r];
    const double idt = 1.0 / D.dyn[R.s].dt;
    const double xi = D.x[r], yi = D.y[r];
    const double rhoi = D.rho[r];
    const double ai = D.qa[r], ipi = D.qi[r];           // rho_i/phi_i, 1/phi_i
    const double wxi = D.qu[r], wyi = D.qw[r];          // vxs_i/phi_i, vys_i/phi_i
    const double bi = ai * ipi;                         // rho_i/phi_i^2
    const double vxsi = D.vxs[r], vysi = D.vys[r];
    const double voli = D.mass[r] / rhoi;
    const double c0 = D.c0[r], c1 = D.c1[r], c2 = D.c2[r], c3 = D.c3[r];
    const bool freei = fl & BS_FLAG_FREE;
    const double lampf = 1.0 / (P.rho * P.rel_den);
    const int n = D.ncount[r];
    const int kmax = D.kmax;
    double dia = 0.0, fv = 0.0;
    for (int k = 0; k < n; ++k) {
        const long e = ell(r, k, kmax);
        const int j = D.nidx[e];
        const double z1 = (double)ld<T>(D.nkx, e), z2 = (double)ld<T>(D.nky, e);
        const double pd = (double)ld<T>(D.nrinv, e);
        const int tj = D.tid[j];
        const double dxi = xi - D.x[j], dyi = yi - D.y[j];
        double off = 0.0;
        if (ti == BS_TID_FLUID) {
            const double lamp = (freei && tj == BS_TID_FLUID) ? (1.0 + D.oden[j] * lampf) : 1.0;
            const double pvol = D.vol[j];
            const double Lx = c0 * z1 + c1 * z2, Ly = c2 * z1 + c3 * z2;
            const double t12 = 2 * pvol * (Lx * dxi + Ly * dyi) * pd;
            off = -t12;
            dia += t12 * lamp;
            double ax, ay;
            if (tj == BS_TID_FLUID) {
                const double aj = D.qa[j];
                const double rho_ij = 2 * aj * ai / (aj + ai);
                ax = rho_ij * (D.qu[j] - wxi);
                ay = rho_ij * (D.qw[j] - wyi);
            } else {
                ax = bi * (D.vxs[j] - vxsi);
                ay = bi * (D.vys[j] - vysi);
            }
            fv += (pvol * (ax * Lx + ay * Ly)) * idt;
        } else if (ti == BS_TID_GHOST) {
            if (tj <= 2) {
                const double t12 = 2 * D.vol[j] * (z1 * dxi + z2 * dyi) * pd;
                off = -t12;
                dia += t12;
            }
        } else if (ti == BS_TID_WALL) {
            if (tj == BS_TID_FLUID) {
                const double d0 = D.c0[j], d1 = D.c1[j], d2 = D.c2[j], d3 = D.c3[j];
                const double Lx = d0 * z1 + d1 * z2, Ly = d2 * z1 + d3 * z2;
                const double t12 = 2 * voli * (Lx * dxi + Ly * dyi) * pd;
                off = -t12;
                dia += t12;
                const double aj = D.qa[j];
                const double ax = aj * (D.qu[j] - vxsi * ipi);
                const double ay = aj * (D.qw[j] - vysi * ipi);
                fv += (voli * (ax * Lx + ay * Ly)) * idt;
            } else {
                const double t12 = 2 * D.vol[j] * (z1 * dxi + z2 * dyi) * pd;
                off = -t12;
                dia += t12;
            }
        }
        st<double>(D.aval, e, off);   // unscaled, scaled below
    }
    // Jacobi scaling (isph.f90:432-440).  A ghost row whose first neighbour
    // is a lower-numbered fluid particle keeps the row initialiser's
    // val(1)=1.0 at col=row (isph.f90:125-128): an extra 1/dia on the diagonal.
    double extra = 0.0;
    if (ti == BS_TID_GHOST && n > 0) {
        const int j0 = D.nidx[ell(r, 0, kmax)];
        if (j0 < r && D.tid[j0] == BS_TID_FLUID) extra = 1.0;
    }
    if (!(dia != 0.0) || !isfinite(dia)) set_err(D, R.s, BS_ERR_ZERO_DIAG);
    const double inv = 1.0 / dia;
    D.adiag[r] = dia / dia + extra * inv;
    D.rhs[r] = fv * inv;
    double* a = (double*)D.aval;
    for (int k = 0; k < n; ++k) {
        const long e = ell(r, k, kmax);
        a[e] = a[e] * inv;
    }
}

// ---------------------------------------------------- comp_vel + comp_pos
// integrator.f90:705-829 and 845-883
template <typename T>
__global__ void __launch_bounds__(BS_THREADS) k_compvel(Dev D, int do_vel, int do_pos) {
    const RowCtx R = row_ctx(D);
    if (!R.active) return;
    const int r = R.r;
    const int ti = D.tid[r];
    const uint8_t fl = D.flags[r];
    const double dt = D.dyn[R.s].dt;
    double vx = D.vx[r], vy = D.vy[r];
    const double phi = D.por[r];
    if (do_vel) {
        double vel = 0.0;
        if (ti == BS_TID_FLUID && !(fl & BS_FLAG_BUFFER)) {
            const T c0 = (T)D.c0[r], c1 = (T)D.c1[r], c2 = (T)D.c2[r], c3 = (T)D.c3[r];
            const double pi = D.p[r], rhoi = D.rho[r];
            const double ai = D.qa[r];   // rho_i/phi_i (k_quot)
            const double qf = 2.0 * (phi * phi) / rhoi;
            const T phi2 = (T)(phi * phi);
            T ax = 0, ay = 0;
            const int n = D.ncount[r];
            const int kmax = D.kmax;
            double axd = 0.0, ayd = 0.0;
            if (sizeof(T) == 4) {
                // mixed: p, rho/phi and the volume of the neighbours from the
                // k_quot records, the pair terms on the FP32 pipe, the
                // pressure-gradient sums (which cancel) compensated
                const float pif = (float)pi, aif = (float)ai, qff = (float)qf, phi2f = (float)(phi * phi);
                const CorrF cf = corr_f(D, r);
                const float rhoif = (float)rhoi;
                Kahan32 kx, ky;
                for (int k = 0; k < n; ++k) {
                    const long e = ell(r, k, kmax);
                    const int j = D.nidx[e];
                    const float z1 = ld<float>(D.nkx, e), z2 = ld<float>(D.nky, e);
                    const float Lx = cf.lx(z1, z2), Ly = cf.ly(z1, z2);
                    const float4 qj = __ldg(D.rec0 + j);   // (p, rho/phi, m/rho)
                    float q;
                    if (D.tid[j] == BS_TID_FLUID) q = qff * qj.z * (qj.x * aif + pif * qj.y) / (aif + qj.y);
                    else q = qj.z * phi2f * (qj.x + pif) / rhoif;
                    kx.add(-(q * Lx));
                    ky.add(-(q * Ly));
                }
                axd = kx.value();
                ayd = ky.value();
            }
            for (int k = 0; k < (sizeof(T) == 4 ? 0 : n); ++k) {
                const long e = ell(r, k, kmax);
                const int j = D.nidx[e];
                const T z1 = ld<T>(D.nkx, e), z2 = ld<T>(D.nky, e);
                const T Lx = c0 * z1 + c1 * z2, Ly = c2 * z1 + c3 * z2;
                const double pj = D.p[j];
                T q;
                if (D.tid[j] == BS_TID_FLUID) {
                    // 2 V_j phi_i^2 (p_j rho_i/phi_i + p_i rho_j/phi_j) / (rho_i (rho_i/phi_i + rho_j/phi_j))
                    const double aj = D.qa[j];
                    q = (T)(qf * D.vol[j] * (pj * ai + pi * aj) / (ai + aj));
                } else {
                    q = (T)D.vol[j] * phi2 * (T)(pj + pi) / (T)rhoi;
                }
                ax -= q * Lx;
                ay -= q * Ly;
            }
            if (sizeof(T) != 4) {
                axd = (double)ax;
                ayd = (double)ay;
            }
            vx = D.vxs[r] + axd * dt;
            vy = D.vys[r] + ayd * dt;
            vel = sqrt(vx * vx + vy * vy) / phi;
            D.vx[r] = vx;
            D.vy[r] = vy;
        } else if (fl & BS_FLAG_BUFFER) {
            vx = D.vxs[r];
            vy = 0.0;
            D.vx[r] = vx;
            D.vy[r] = vy;
        }
        D.vel[r] = vel;
    }
    if (do_pos && ti == BS_TID_FLUID) {
        // x = (x + xs + dt*vx/porosity)/2 (integrator.f90:859-863), no FMA
        const double x = D.x[r], y = D.y[r];
        const double xn = __ddiv_rn(__dadd_rn(__dadd_rn(x, D.xs[r]), __ddiv_rn(__dmul_rn(dt, vx), phi)), 2.0);
        const double yn = __ddiv_rn(__dadd_rn(__dadd_rn(y, D.ys[r]), __ddiv_rn(__dmul_rn(dt, vy), phi)), 2.0);
        D.x[r] = xn;
        D.y[r] = yn;
        // buffer release (integrator.f90:865-872)
        const ScenePar& P = D.par[R.s];
        if ((fl & BS_FLAG_BUFFER) && (xn > P.buf_lo) && (xn < P.buf_hi)) D.flags[r] = fl & ~BS_FLAG_BUFFER;
    }
}

// ------------------------------------------------------------ opt2_shift
// part_shift.f90:12-169 (shift and Taylor velocity correction; applied by
// k_apply_density).  The free-surface normals are forced to zero (67-68)
// and pint = 0 (69), so the shift uses the raw kernel gradient.
template <typename T>
__global__ void __launch_bounds__(BS_THREADS) k_shift(Dev D) {
    const RowCtx R = row_ctx(D);
    if (!R.active) return;
    const ScenePar& P = D.par[R.s];
    const int r = R.r;
    const uint8_t fl = D.flags[r];
    if (D.tid[r] != BS_TID_FLUID || (fl & BS_FLAG_BUFFER)) return;
    const int n = D.ncount[r];
    if (n == 0) {   // keeps stale xs/ys/vxs/vys, as the reference (part_shift.f90:39)
        set_err(D, R.s, BS_ERR_NO_NEIGHBOUR);
        return;
    }
    const T c0 = (T)D.c0[r], c1 = (T)D.c1[r], c2 = (T)D.c2[r], c3 = (T)D.c3[r];
    const double vxi = D.vx[r], vyi = D.vy[r];
    T sxs = 0, sys = 0, a1 = 0, a2 = 0, b1 = 0, b2 = 0;
    const int kmax = D.kmax;
    if (sizeof(T) == 4) {
        // mixed: the neighbours' velocities as (hi, lo) pairs and volumes
        // from the k_quot records, the differences rounded once to FP32
        const float4 vi4 = D.rec0[r];
        const CorrF cf = corr_f(D, r);
        for (int k = 0; k < n; ++k) {
            const long e = ell(r, k, kmax);
            const int j = D.nidx[e];
            const float z1 = ld<float>(D.nkx, e), z2 = ld<float>(D.nky, e);
            const float V = __ldg(D.rec1 + j).x;
            sxs += z1 * V;
            sys += z2 * V;
            const float Lx = cf.lx(z1, z2), Ly = cf.ly(z1, z2);
            const float4 vj4 = __ldg(D.rec0 + j);
            const float du = f2_diff(vj4.x, vj4.y, vi4.x, vi4.y).x, dv = f2_diff(vj4.z, vj4.w, vi4.z, vi4.w).x;
            a1 += Lx * du * V;
            a2 += Ly * du * V;
            b1 += Lx * dv * V;
            b2 += Ly * dv * V;
        }
    }
    for (int k = 0; k < (sizeof(T) == 4 ? 0 : n); ++k) {
        const long e = ell(r, k, kmax);
        const int j = D.nidx[e];
        const T z1 = ld<T>(D.nkx, e), z2 = ld<T>(D.nky, e);
        const T V = (T)D.vol[j];
        sxs += z1 * V;
        sys += z2 * V;
        const T Lx = c0 * z1 + c1 * z2, Ly = c2 * z1 + c3 * z2;
        const T du = (T)(D.vx[j] - vxi), dv = (T)(D.vy[j] - vyi);
        a1 += Lx * du * V;
        a2 += Ly * du * V;
        b1 += Lx * dv * V;
        b2 += Ly * dv * V;
    }
    const double frac = (fl & BS_FLAG_FREE) ? 0.01 : 1.0;
    const double cfac = -P.csh * (P.h * P.h) * frac;
    const double xs = cfac * (double)sxs, ys = cfac * (double)sys;
    const double cap = P.maxshift * P.dl;
    if (sizeof(T) == 4) {
        // mixed form: a component of the FP32 sum that cancels to exactly 0
        // (a neighbourhood symmetric along that axis) is no shift along it;
        // the FP64 drop-in keeps the reference's 0 * 0 / 0 below
        D.xs[r] = xs == 0.0 ? 0.0 : fmin(fabs(xs), cap) * xs / fabs(xs);
        D.ys[r] = ys == 0.0 ? 0.0 : fmin(fabs(ys), cap) * ys / fabs(ys);
    } else {
        if (xs == 0.0 || ys == 0.0) set_err(D, R.s, BS_ERR_ZERO_SHIFT);
        D.xs[r] = fmin(fabs(xs), cap) * xs / fabs(xs);
        D.ys[r] = fmin(fabs(ys), cap) * ys / fabs(ys);
    }
    D.vxs[r] = (double)a1 * xs + (double)a2 * ys;
    D.vys[r] = (double)b1 * xs + (double)b2 * ys;
}

// apply the shift (part_shift.f90:172-189) and densityupdate (scalar.f90:399-426)
__global__ void k_apply_density(Dev D, int do_apply, int do_density) {
    const RowCtx R = row_ctx(D);
    if (!R.active) return;
    const ScenePar& P = D.par[R.s];
    const int r = R.r;
    if (D.tid[r] != BS_TID_FLUID) return;
    const uint8_t fl = D.flags[r];
    if (do_apply && !(fl & BS_FLAG_BUFFER)) {
        const double x = __dadd_rn(D.x[r], D.xs[r]), y = __dadd_rn(D.y[r], D.ys[r]);
        D.x[r] = x;
        D.y[r] = y;
        D.vx[r] = D.vx[r] + D.vxs[r];
        D.vy[r] = D.vy[r] + D.vys[r];
    }
    if (do_density) {
        const double od = 0.5 * (P.rhomax + P.rhomin) + D.con[r] * (P.rhomax - P.rhomin);
        const double m = od * D.ovol[r];
        const double rh = od * D.por[r];
        D.oden[r] = od;
        D.mass[r] = m;
        D.rho[r] = rh;
        D.vol[r] = m / rh;
        D.nu[r] = bs_vis(od) / od;
    }
}

// |v|/porosity for fluid rows (the vel of comp_vel, integrator.f90:814-815),
// from the uploaded velocities: initial timestep maxima
__global__ void k_velmag(Dev D) {
    const RowCtx R = row_ctx(D);
    if (!R.active) return;
    const int r = R.r;
    double v = 0.0;
    if (D.tid[r] == BS_TID_FLUID && !(D.flags[r] & BS_FLAG_BUFFER)) {
        const double vx = D.vx[r], vy = D.vy[r];
        v = sqrt(vx * vx + vy * vy) / D.por[r];
    }
    D.vel[r] = v;
}

// dispersion tensor per particle (scalar.f90:267-301), for the stand-alone
// scalar entry point (the fused step computes it in the final k_eddy)
__global__ void k_disp(Dev D) {
    const RowCtx R = row_ctx(D);
    if (!R.active) return;
    const ScenePar& P = D.par[R.s];
    const int r = R.r;
    if (D.tid[r] != BS_TID_FLUID) return;
    const double al = 0.0025, at = 0.00025, Dm = BS_SP1EM9;
    const double vx = D.vx[r], vy = D.vy[r], phi = D.por[r];
    const double vi = sqrt(vx * vx + vy * vy) / phi;
    const double dl_ = sqrt((al * vi) + Dm) * vi * phi, dt_ = sqrt((at * vi) + Dm) * vi * phi;
    D.Dp0[r] = vx / dl_;
    D.Dp1[r] = vy / dl_;
    D.Dp2[r] = (-vy) / dt_;
    D.Dp3[r] = vx / dt_;
    D.Dt[r] = Dm + D.nut[r] / P.tschmidt;
}

// ------------------------------------------------------------- scalar
// scalart_anisotropic (scalar.f90:242-362) + scalarupdate (364-397); reads
// con, writes con_new (swapped by the host).  Uses the stored pair distance
// with the current positions, as the reference does.
template <typename T>
__global__ void __launch_bounds__(BS_THREADS) k_scalar(Dev D, int substep, const int* jdev) {
    const RowCtx R = row_ctx(D);
    if (!R.active) return;
    if (jdev) substep += *jdev;   // the captured step counts its sub-step pairs on the device
    const ScenePar& P = D.par[R.s];
    const int r = R.r;
    const double coni = D.con[r];
    // sub-steps beyond this scene's solsteps (integrator.f90:941-949) copy through
    if (D.tid[r] != BS_TID_FLUID || !P.scalar_on || substep >= D.dyn[R.s].solsteps) {
        D.con_new[r] = coni;
        return;
    }
    const double thr = 0.7;
    const double phii = D.por[r], nuti = D.nut[r];
    const double xi = D.x[r], yi = D.y[r];
    const double Pi0 = D.Dp0[r], Pi1 = D.Dp1[r], Pi2 = D.Dp2[r], Pi3 = D.Dp3[r], Dti = D.Dt[r];
    const double cap = 0.12 * (P.dl * P.dl) / D.dyn[R.s].dt;
    const double ovoli = D.ovol[r];
    double cd = 0.0;
    const int n = D.ncount[r];
    const int kmax = D.kmax;
    if (sizeof(T) == 4) {
        // mixed: the pair terms in FP32 from the FP32-stored pair data and the
        // k_quot records (dispersion tensor, Dt, con, phi; the porosity and
        // eddy-viscosity thresholds as flags taken on the FP64 values; the
        // pair offset from the double-float positions), summed in FP32
        const float capf = (float)cap, ovf = (float)ovoli, phif = (float)phii, cof = (float)coni;
        const float P0 = (float)Pi0, P1 = (float)Pi1, P2 = (float)Pi2, P3 = (float)Pi3, Dtf = (float)Dti;
        const bool nsmall = nuti < BS_SP1EM6, psmall = phii < thr;
        const float4 pi4 = D.pos4[r];
        const KerF KF = ker_f(P);
        float cdf = 0.0f;
        for (int k = 0; k < n; ++k) {
            const long e = ell(r, k, kmax);
            const int j = D.nidx[e];
            if (D.tid[j] != BS_TID_FLUID) continue;
            const float4 sj = __ldg(D.rec1 + j);   // (Dt, con, phi, flags)
            const int bits = (int)sj.w;
            const float pj = sj.z;
            const float dm = ld<float>(D.ndist, e);
            const float4 pj4 = __ldg(D.pos4 + j);
            const float dx = f2_diff(pi4.x, pi4.y, pj4.x, pj4.y).x, dy = f2_diff(pi4.z, pi4.w, pj4.z, pj4.w).x;
            float t1x;
            if (psmall && (bits & 1)) {
                const float4 dj = __ldg(D.rec0 + j);
                const float Dxx = P0 + dj.x, Dxy = P1 + dj.y;
                const float Dyx = P2 + dj.z, Dyy = P3 + dj.w;
                const float ph = 0.5f / dm;
                const float A = Dxx * dx * ph + Dxy * dy * ph, B = Dyx * dx * ph + Dyy * dy * ph;
                t1x = 1.0f / (A * A + B * B);
                t1x = (t1x <= capf) ? t1x : capf;
            } else {
                const float Dj = sj.x;
                if (nsmall && (bits & 2)) t1x = (Dtf + Dj) * 0.5f;
                else t1x = 2.0f * Dtf * Dj / (Dtf + Dj);
            }
            const float t3 = ovf * (phif + pj) / (phif * pj);
            const float F = bs_Ff(dm, KF);
            const float pd = ld<float>(D.nrinv, e);
            const float dc = cof - sj.y;
            cdf += t1x * t3 * dc * (dx * (F * dx) + dy * (F * dy)) * pd;
        }
        cd = cdf;
    }
    for (int k = 0; k < (sizeof(T) == 4 ? 0 : n); ++k) {
        const long e = ell(r, k, kmax);
        const int j = D.nidx[e];
        if (D.tid[j] != BS_TID_FLUID) continue;
        const double phij = D.por[j];
        const bool pz = (phii < thr) && (phij < thr);
        const double dm = (double)ld<T>(D.ndist, e);
        const double dxi = xi - D.x[j], dyi = yi - D.y[j];
        double t1x;
        if (pz) {
            const double Dxx = Pi0 + D.Dp0[j], Dxy = Pi1 + D.Dp1[j], Dyx = Pi2 + D.Dp2[j], Dyy = Pi3 + D.Dp3[j];
            const double pdist = 1.0 / dm;
            const double A = (Dxx * dxi * pdist * 0.5) + (Dxy * dyi * pdist * 0.5);
            const double B = (Dyx * dxi * pdist * 0.5) + (Dyy * dyi * pdist * 0.5);
            t1x = 1.0 / (A * A + B * B);
            t1x = (t1x <= cap) ? t1x : cap;
        } else {
            const double Dxxj = D.Dt[j];
            if ((nuti < BS_SP1EM6) && (D.nut[j] < BS_SP1EM6)) t1x = (Dti + Dxxj) * 0.50;
            else t1x = 2 * Dti * Dxxj / (Dti + Dxxj);
        }
        const double t3 = ovoli * (phii + phij) / (phii * phij);
        const double F = bs_F(dm, P);
        const double pd = (double)ld<T>(D.nrinv, e);
        const double dc = coni - D.con[j];
        cd += (t1x * t3 * dc * dxi * (F * dxi) * pd) + (t1x * t3 * dc * dyi * (F * dyi) * pd);
    }
    D.cdiff[r] = cd;
    double cn = coni + cd * D.dyn[R.s].dtsol;
    if ((D.flags[r] & BS_FLAG_BUFFER) && (xi < 1.6)) cn = 0.5;
    D.con_new[r] = cn;
}

}  // namespace

namespace bs {

// ------------------------------------------------------------------ WCSPH
// wcsph.f90, a module the reference ships but never calls.

// hydrostatic Tait density at height y (the term2 expression, wcsph.f90:78-82)
__device__ __forceinline__ double wc_hyd(const ScenePar& P, double y) {
    const double rho = P.rho, co = P.wc_c0, gam = P.wc_gamma;
    return rho * pow(((((P.wc_ysurf - y) * rho) * fabs(P.g)) * gam) / (rho * (co * co)) + 1.0, 1.0 / gam);
}

// per-row hydrostatic density (one pow per particle, not per pair)
__global__ void k_wc_hyd(Dev D) {
    const RowCtx R = row_ctx(D);
    if (!R.active) return;
    D.whyd[R.r] = wc_hyd(D.par[R.s], D.y[R.r]);
}

// calmasscons, wcsph.f90:65-129, for fluid rows: tden = rho + dt * (term1 +
// term2), the L-corrected velocity divergence plus delta-SPH diffusion with
// the hydrostatic correction.  As written (wc_form 0) term2 is also the
// pair's hydrostatic difference and is overwritten by it at every
// neighbour, so only the last neighbour's y contribution survives, and the
// delta-SPH term runs along (r_i - r_j), which makes it anti-diffusive;
// wc_form 1 sums the y terms over all neighbours and takes (r_j - r_i).
template <typename T>
__global__ void __launch_bounds__(BS_THREADS) k_wc_continuity(Dev D) {
    const RowCtx R = row_ctx(D);
    if (!R.active) return;
    const int r = R.r;
    if (!(D.tid[r] > 2)) return;
    const ScenePar& P = D.par[R.s];
    const double co = P.wc_c0, delt = P.wc_delta, h1 = P.h, lam = P.lam;
    const double dt = D.dyn[R.s].dt;
    const double xi = D.x[r], yi = D.y[r], vxi = D.vx[r], vyi = D.vy[r], rhoi = D.rho[r];
    const double c0 = D.c0[r], c1 = D.c1[r], c2 = D.c2[r], c3 = D.c3[r];
    const double hydi = D.whyd[r];
    const double dfac = ((delt * 2) * h1) * co;
    double term1 = 0.0, term2 = 0.0;
    const int n = D.ncount[r];
    if (sizeof(T) == 4) {
        // mixed: the neighbours' velocities, densities and hydrostatic
        // densities as (hi, lo) pairs and masses from the k_quot records, the
        // pair offsets from the double-float positions, each cancelling
        // difference rounded once to FP32; the pair terms on the FP32 pipe,
        // the sums compensated
        const float4 pi4 = D.pos4[r], vi4 = D.rec0[r], di4 = D.rec1[r];
        const CorrF cf = corr_f(D, r);
        const float dfacf = (float)dfac, lamf = (float)lam, rhoif = di4.x;
        const float sg = (P.wc_form == 0) ? 1.0f : -1.0f;
        Kahan32 k1, k2;
        for (int k = 0; k < n; ++k) {
            const long e = ell(r, k, D.kmax);
            const int j = D.nidx[e];
            const float rad = ld<float>(D.ndist, e);
            const float wx = ld<float>(D.nkx, e), wy = ld<float>(D.nky, e);
            const float4 dj4 = __ldg(D.rec1 + j), vj4 = __ldg(D.rec0 + j), pj4 = __ldg(D.pos4 + j);
            const float hd = f2_diff(dj4.z, dj4.w, di4.z, di4.w).x;
            if (P.wc_form == 0) k2 = Kahan32{hd, 0.0f};
            const float gx = cf.lx(wx, wy);
            const float gy = cf.ly(wx, wy);
            const float mj = __ldg(D.rec2 + j).x, rhoj = dj4.x;
            const float vr = mj / rhoj, den = rad * rad + lamf;
            const float drho = f2_diff(dj4.x, dj4.y, di4.x, di4.y).x - hd;
            const float dxi = f2_diff(pi4.x, pi4.y, pj4.x, pj4.y).x, dyi = f2_diff(pi4.z, pi4.w, pj4.z, pj4.w).x;
            const float dvx = f2_diff(vj4.x, vj4.y, vi4.x, vi4.y).x, dvy = f2_diff(vj4.z, vj4.w, vi4.z, vi4.w).x;
            k1.add(-(((mj * dvx) * gx) * (rhoif / rhoj)) + (((dfacf * drho) * (sg * dxi)) * gx) * vr / den);
            k2.add(-(((mj * dvy) * gy) * (rhoif / rhoj)) + (((dfacf * drho) * (sg * dyi)) * gy) * vr / den);
        }
        D.tden[r] = rhoi + (k1.value() + k2.value()) * dt;
        return;
    }
    for (int k = 0; k < n; ++k) {
        const long e = ell(r, k, D.kmax);
        const int j = D.nidx[e];
        const double rad = (double)ld<T>(D.ndist, e);
        const double wx = (double)ld<T>(D.nkx, e), wy = (double)ld<T>(D.nky, e);
        const double hd = D.whyd[j] - hydi;
        // as written: term2 doubles as the hydrostatic difference and the
        // delta term runs along (r_i - r_j) (anti-diffusive); corrected:
        // own y sum, delta term along (r_j - r_i)
        const double sg = (P.wc_form == 0) ? 1.0 : -1.0;
        if (P.wc_form == 0) term2 = hd;
        const double gx = c0 * wx + c1 * wy;
        const double gy = c2 * wx + c3 * wy;
        const double mj = D.mass[j], rhoj = D.rho[j];
        const double vr = mj / rhoj, den = rad * rad + lam;
        term1 = term1 - ((mj * (D.vx[j] - vxi)) * gx) * (rhoi / rhoj) +
                (((dfac * (rhoj - rhoi - hd)) * (sg * (xi - D.x[j]))) * gx) * vr / den;
        term2 = term2 - ((mj * (D.vy[j] - vyi)) * gy) * (rhoi / rhoj) +
                (((dfac * (rhoj - rhoi - hd)) * (sg * (yi - D.y[j]))) * gy) * vr / den;
    }
    D.tden[r] = rhoi + (term1 + term2) * dt;
}

// per-row WCSPH updates: bit0 updateden (wcsph.f90:131-154), bit1
// dentopress (Tait, wcsph.f90:35-63), bit2 presstoden (wcsph.f90:13-33);
// the derived volume m/rho follows the density
__global__ void k_wc_rows(Dev D, int mode) {
    const RowCtx R = row_ctx(D);
    if (!R.active) return;
    const int r = R.r;
    const ScenePar& P = D.par[R.s];
    const double rho = P.rho, co = P.wc_c0, gam = P.wc_gamma;
    double d = D.rho[r];
    const bool fluid = D.tid[r] > 2;
    if ((mode & 1) && fluid) d = D.tden[r];
    if ((mode & 2) && fluid) {
        double p = (rho * (co * co)) * (pow(d / rho, gam) - 1) / gam;
        if (p < 0.0) {
            p = 0.0;
            d = rho;
        }
        D.p[r] = p;
    }
    if (mode & 4) d = rho * pow((D.p[r] * gam / (rho * (co * co))) + 1, 1 / gam);
    if (d != D.rho[r]) {
        D.rho[r] = d;
        D.vol[r] = D.mass[r] / d;
    }
}

// wall and ghost pressure of the WCSPH step (this library's boundary rule):
// Shepard average over fluid neighbours of p_f + rho_f |g| (y_f - y_w)
template <typename T>
__global__ void __launch_bounds__(BS_THREADS) k_wc_wallp(Dev D) {
    const RowCtx R = row_ctx(D);
    if (!R.active) return;
    const int r = R.r;
    if (D.tid[r] == BS_TID_FLUID) return;
    const ScenePar& P = D.par[R.s];
    const double ag = fabs(P.g), yw = D.y[r];
    double num = 0.0, den = 0.0;
    const int n = D.ncount[r];
    for (int k = 0; k < n; ++k) {
        const long e = ell(r, k, D.kmax);
        const int j = D.nidx[e];
        if (D.tid[j] != BS_TID_FLUID) continue;
        const double w = bs_W((double)ld<T>(D.ndist, e), P);
        num += (D.p[j] + D.rho[j] * ag * (D.y[j] - yw)) * w;
        den += w;
    }
    D.p[r] = den > 0.0 ? num / den : 0.0;
}

// ------------------------------------------------ wall / ghost velocity
// boun_vel (integrator.f90:394-457, compiled but never called) and
// comp_ghost + ghost_en (mls.f90:114-263, not compiled): wall and ghost rows
// take minus the Shepard average of their fluid neighbours (no-slip mirror);
// products in the reference's evaluation order, no contraction.
template <typename T>
__global__ void __launch_bounds__(BS_THREADS) k_boun_vel(Dev D) {
    const RowCtx R = row_ctx(D);
    if (!R.active) return;
    const int r = R.r;
    if (D.tid[r] > 2) return;
    const ScenePar& P = D.par[R.s];
    double vx = 0.0, vy = 0.0, t1 = 0.0;
    const int n = D.ncount[r];
    for (int k = 0; k < n; ++k) {
        const long e = ell(r, k, D.kmax);
        const int j = D.nidx[e];
        if (D.tid[j] != BS_TID_FLUID) continue;
        const double w = bs_W((double)ld<T>(D.ndist, e), P);
        const double mw = __dmul_rn(D.mass[j], w), rj = D.rho[j];
        vx = __dsub_rn(vx, __ddiv_rn(__dmul_rn(mw, D.vx[j]), rj));
        vy = __dsub_rn(vy, __ddiv_rn(__dmul_rn(mw, D.vy[j]), rj));
        t1 = __dadd_rn(t1, __ddiv_rn(mw, rj));
    }
    if (t1 >= BS_SP1EM6) {
        vx = __ddiv_rn(vx, t1);
        vy = __ddiv_rn(vy, t1);
    }
    D.vx[r] = vx;
    D.vy[r] = vy;
    D.vxs[r] = 0.0;
    D.vys[r] = 0.0;
}

// ------------------------------------------------ collision shifts
// coll_pos_shift (mode 0, part_shift.f90:193-292) and coll_shift (mode 1,
// 294-410), compiled but never called.  Pass 1 (k_coll): every row's xs, ys
// (mode 0) or vxs, vys (mode 1) zeroed; for fluid rows with neighbours,
// gradvx >= 0.7 and not in a buffer, per axis t1 = sum m_j and t2 = sum of
// the pushes of the neighbours closer than
// dcol = pr/sqrt(phi_i) + (fluid_j ? pr : br)/sqrt(phi_j); the shift is
// t2 / (m_i + t1).  The push is -(m_j (1 + cr) (d - dcol)) (x_i - x_j)/d
// (mode 0) or, where the relative pore velocity approaches (t3 < 0),
// -(m_j (1 + cr) t3) (x_i - x_j)/d^2 (mode 1); cr = 0.  Pass 2
// (k_coll_apply) moves or accelerates the rows after every shift is known.
// Products in the reference's evaluation order, no contraction; a failed
// condition adds 0.0 as merge() does.
template <typename T>
__global__ void __launch_bounds__(BS_THREADS) k_coll(Dev D, int mode, double prx, double pry, double brx,
                                                     double bry) {
    const RowCtx R = row_ctx(D);
    if (!R.active) return;
    const int r = R.r;
    double* sxp = mode ? D.vxs : D.xs;
    double* syp = mode ? D.vys : D.ys;
    const int n = D.ncount[r];
    if (!(n != 0 && D.gradvx[r] >= 0.70 && D.tid[r] == BS_TID_FLUID && !(D.flags[r] & BS_FLAG_BUFFER))) {
        sxp[r] = 0.0;
        syp[r] = 0.0;
        return;
    }
    const double cr = 0.0, disfac = 1.0;
    const double xi = D.x[r], yi = D.y[r], phi = D.por[r], mi = D.mass[r];
    const double isq = __ddiv_rn(1.0, __dsqrt_rn(phi)), iphi = __ddiv_rn(1.0, phi);
    const double vxi = __dmul_rn(D.vx[r], iphi), vyi = __dmul_rn(D.vy[r], iphi);
    double out[2];
    for (int ax = 0; ax < 2; ++ax) {
        const double pr = ax ? pry : prx, br = ax ? bry : brx;
        double t1 = 0.0, t2 = 0.0;
        for (int k = 0; k < n; ++k) {
            const long e = ell(r, k, D.kmax);
            const int j = D.nidx[e];
            const double d = (double)ld<T>(D.ndist, e);
            const double phj = D.por[j];
            const double dcol = __dmul_rn(disfac, __dadd_rn(__dmul_rn(pr, isq),
                __dmul_rn(D.tid[j] == BS_TID_FLUID ? pr : br, __ddiv_rn(1.0, __dsqrt_rn(phj)))));
            const double mj = D.mass[j];
            t1 = __dadd_rn(t1, mj);
            const double rel = ax ? __dsub_rn(yi, D.y[j]) : __dsub_rn(xi, D.x[j]);
            double term = 0.0;
            if (mode == 0) {
                if (d < dcol)
                    term = __dmul_rn(__dmul_rn(-1.0, __dmul_rn(__dmul_rn(mj, 1.0 + cr), __dsub_rn(d, dcol))),
                                     __ddiv_rn(rel, d));
            } else {
                const double iphj = __ddiv_rn(1.0, phj);
                const double t3 = __dadd_rn(
                    __dmul_rn(__dsub_rn(xi, D.x[j]), __dsub_rn(vxi, __dmul_rn(D.vx[j], iphj))),
                    __dmul_rn(__dsub_rn(yi, D.y[j]), __dsub_rn(vyi, __dmul_rn(D.vy[j], iphj))));
                if (d < dcol && t3 < 0.0)
                    term = __dmul_rn(__dmul_rn(-1.0, __dmul_rn(__dmul_rn(mj, 1.0 + cr), t3)),
                                     __ddiv_rn(rel, __dmul_rn(d, d)));
            }
            t2 = __dadd_rn(t2, term);
        }
        out[ax] = __ddiv_rn(t2, __dadd_rn(mi, t1));
    }
    sxp[r] = out[0];
    syp[r] = out[1];
}

__global__ void __launch_bounds__(BS_THREADS) k_coll_apply(Dev D, int mode) {
    const RowCtx R = row_ctx(D);
    if (!R.active) return;
    const int r = R.r;
    if (D.tid[r] != BS_TID_FLUID || (D.flags[r] & BS_FLAG_BUFFER)) return;
    if (mode == 0) {
        if (D.gradvx[r] >= 0.70) {
            const double x = __dadd_rn(D.x[r], D.xs[r]), y = __dadd_rn(D.y[r], D.ys[r]);
            D.x[r] = x;
            D.y[r] = y;
        }
    } else {
        D.vx[r] = __dadd_rn(D.vx[r], __dmul_rn(D.vxs[r], D.por[r]));
        D.vy[r] = __dadd_rn(D.vy[r], __dmul_rn(D.vys[r], D.por[r]));
    }
}

// use_mls: the velocity by the module's commented-out moving-least-squares
// branch, weights W (b1 + b2 dx + b3 dy) V, b = first column of the inverse
// of the moment matrix over all neighbours (Wmls, mls.f90:16-111;
// invertmat3D, functions.f90:134-165), where its determinant reaches 1e-5
// (single literal); the Shepard average elsewhere.  tke and nut always by
// Shepard (ghost_en).  A zero Shepard sum leaves 0.
template <typename T>
__global__ void __launch_bounds__(BS_THREADS) k_ghost(Dev D, int use_mls) {
    const RowCtx R = row_ctx(D);
    if (!R.active) return;
    const int r = R.r;
    if (D.tid[r] > 2) return;
    const ScenePar& P = D.par[R.s];
    const int n = D.ncount[r];
    const double xi = D.x[r], yi = D.y[r];
    double vx = 0.0, vy = 0.0, tke = 0.0, nut = 0.0;
    bool err = true;
    double b0 = 0.0, b1 = 0.0, b2 = 0.0;
    if (n > 0 && use_mls) {
        double a00 = 0, a10 = 0, a20 = 0, a01 = 0, a11 = 0, a21 = 0, a02 = 0, a12 = 0, a22 = 0;
        for (int k = 0; k < n; ++k) {
            const long e = ell(r, k, D.kmax);
            const int j = D.nidx[e];
            const double w = bs_W((double)ld<T>(D.ndist, e), P);
            const double v = __ddiv_rn(D.mass[j], D.rho[j]);
            const double dx = __dsub_rn(xi, D.x[j]), dy = __dsub_rn(yi, D.y[j]);
            const double wdx = __dmul_rn(w, dx), wdy = __dmul_rn(w, dy);
            a00 = __dadd_rn(a00, __dmul_rn(w, v));
            a10 = __dadd_rn(a10, __dmul_rn(wdx, v));
            a20 = __dadd_rn(a20, __dmul_rn(wdy, v));
            a01 = __dadd_rn(a01, __dmul_rn(wdx, v));
            a11 = __dadd_rn(a11, __dmul_rn(__dmul_rn(w, __dmul_rn(dx, dx)), v));
            a21 = __dadd_rn(a21, __dmul_rn(__dmul_rn(wdx, dy), v));
            a02 = __dadd_rn(a02, __dmul_rn(wdy, v));
            a12 = __dadd_rn(a12, __dmul_rn(__dmul_rn(wdx, dy), v));
            a22 = __dadd_rn(a22, __dmul_rn(__dmul_rn(w, __dmul_rn(dy, dy)), v));
        }
        auto mul = [](double a, double b) { return __dmul_rn(a, b); };
        auto sub = [](double a, double b) { return __dsub_rn(a, b); };
        const double det = __dadd_rn(__dsub_rn(mul(a00, sub(mul(a11, a22), mul(a21, a12))),
                                               mul(a01, sub(mul(a10, a22), mul(a20, a12)))),
                                     mul(a02, sub(mul(a10, a21), mul(a20, a11))));
        if (!(det < (double)1e-5f) && isfinite(det)) {
            err = false;
            b0 = __ddiv_rn(sub(mul(a11, a22), mul(a21, a12)), det);
            b1 = __ddiv_rn(-sub(mul(a01, a22), mul(a21, a02)), det);
            b2 = __ddiv_rn(sub(mul(a01, a12), mul(a11, a02)), det);
        }
    }
    double t1 = 0.0, te = 0.0;
    for (int k = 0; k < n; ++k) {
        const long e = ell(r, k, D.kmax);
        const int j = D.nidx[e];
        if (D.tid[j] != BS_TID_FLUID) continue;
        const double w = bs_W((double)ld<T>(D.ndist, e), P);
        const double mj = D.mass[j], rj = D.rho[j];
        if (!err) {
            const double corr = __dadd_rn(__dadd_rn(b0, __dmul_rn(b1, __dsub_rn(xi, D.x[j]))),
                                          __dmul_rn(b2, __dsub_rn(yi, D.y[j])));
            const double q = __dmul_rn(__dmul_rn(w, corr), __ddiv_rn(mj, rj));
            vx = __dsub_rn(vx, __dmul_rn(D.vx[j], q));
            vy = __dsub_rn(vy, __dmul_rn(D.vy[j], q));
        } else {
            vx = __dsub_rn(vx, __ddiv_rn(__dmul_rn(__dmul_rn(w, D.vx[j]), mj), rj));
            vy = __dsub_rn(vy, __ddiv_rn(__dmul_rn(__dmul_rn(w, D.vy[j]), mj), rj));
            t1 = __dadd_rn(t1, __ddiv_rn(__dmul_rn(mj, w), rj));
        }
        tke = __dsub_rn(tke, __ddiv_rn(__dmul_rn(__dmul_rn(w, D.tke[j]), mj), rj));
        nut = __dsub_rn(nut, __ddiv_rn(__dmul_rn(__dmul_rn(w, D.nut[j]), mj), rj));
        te = __dadd_rn(te, __ddiv_rn(__dmul_rn(mj, w), rj));
    }
    if (err && t1 > 0.0) {
        vx = __ddiv_rn(vx, t1);
        vy = __ddiv_rn(vy, t1);
    }
    if (te > 0.0) {
        tke = __ddiv_rn(tke, te);
        nut = __ddiv_rn(nut, te);
    }
    D.vx[r] = vx;
    D.vy[r] = vy;
    D.tke[r] = tke;
    D.nut[r] = nut;
}

#define BS_DISPATCH(id, prec, kern, ...)                                                          \
    do {                                                                                          \
        const int q_ = tbegin(L, id);                                                             \
        if ((prec) == BS_PREC_MIXED)                                                              \
            kern<float><<<row_blocks(L, L.sweep_tpb), L.sweep_tpb, 0, L.stream>>>(__VA_ARGS__);   \
        else kern<double><<<row_blocks(L, L.sweep_tpb), L.sweep_tpb, 0, L.stream>>>(__VA_ARGS__); \
        tend(L, q_);                                                                              \
    } while (0)
#define BS_PLAIN(id, kern, ...)                                                                   \
    do {                                                                                          \
        const int q_ = tbegin(L, id);                                                             \
        kern<<<row_blocks(L, L.sweep_tpb), L.sweep_tpb, 0, L.stream>>>(__VA_ARGS__);              \
        tend(L, q_);                                                                              \
    } while (0)

void search(const Dev& D, const Launch& L, int precision, int do_search, int do_effpor) {
    BS_PLAIN(K_RELPOS, k_relpos, D);
    BS_DISPATCH(K_SEARCH, precision, k_search, D, do_search, do_effpor);
}
void freesurf(const Dev& D, const Launch& L) { BS_PLAIN(K_FREESURF, k_freesurf, D); }
void eddy(const Dev& D, const Launch& L, int precision, int with_eddy, int with_varts, int with_disp) {
    BS_PLAIN(K_EDDY, k_quot, D, 1);
    BS_DISPATCH(K_EDDY, precision, k_eddy, D, with_eddy, with_varts, with_disp);
}
void int_vel(const Dev& D, const Launch& L, int precision) {
    if (precision == BS_PREC_MIXED) BS_PLAIN(K_INTVEL, k_quot, D, 3);
    BS_DISPATCH(K_INTVEL, precision, k_intvel, D);
}
void assemble(const Dev& D, const Launch& L, int precision) {
    BS_PLAIN(K_ASSEMBLE, k_quot, D, 0);
    BS_DISPATCH(K_ASSEMBLE, precision, k_assemble, D);
}
void comp_vel(const Dev& D, const Launch& L, int precision, int do_vel, int do_pos) {
    if (do_vel) BS_PLAIN(K_COMPVEL, k_quot, D, 2);
    BS_DISPATCH(K_COMPVEL, precision, k_compvel, D, do_vel, do_pos);
}
void shift(const Dev& D, const Launch& L, int precision) {
    if (precision == BS_PREC_MIXED) BS_PLAIN(K_SHIFT, k_quot, D, 5);
    BS_DISPATCH(K_SHIFT, precision, k_shift, D);
}
void apply_density(const Dev& D, const Launch& L, int do_apply, int do_density) {
    BS_PLAIN(K_APPLY, k_apply_density, D, do_apply, do_density);
}
void disp(const Dev& D, const Launch& L) { BS_PLAIN(K_DISP, k_disp, D); }
void velmag(const Dev& D, const Launch& L) { BS_PLAIN(K_VELMAG, k_velmag, D); }
void scalar(const Dev& D, const Launch& L, int precision, int substep, const int* jdev) {
    if (precision == BS_PREC_MIXED) BS_PLAIN(K_SCALAR, k_quot, D, 4);
    BS_DISPATCH(K_SCALAR, precision, k_scalar, D, substep, jdev);
}
void wc_continuity(const Dev& D, const Launch& L, int precision) {
    BS_PLAIN(K_WC_CONT, k_wc_hyd, D);
    if (precision == BS_PREC_MIXED) BS_PLAIN(K_WC_CONT, k_quot, D, 6);
    BS_DISPATCH(K_WC_CONT, precision, k_wc_continuity, D);
}
void wc_rows(const Dev& D, const Launch& L, int mode) { BS_PLAIN(K_WC_ROWS, k_wc_rows, D, mode); }
void wc_wall_pressure(const Dev& D, const Launch& L, int precision) {
    BS_DISPATCH(K_WC_WALLP, precision, k_wc_wallp, D);
}

void boun_vel(const Dev& D, const Launch& L, int precision) { BS_DISPATCH(K_GHOST, precision, k_boun_vel, D); }
void collision_shift(const Dev& D, const Launch& L, int precision, int mode, double prx, double pry, double brx,
                     double bry) {
    BS_DISPATCH(K_COLL, precision, k_coll, D, mode, prx, pry, brx, bry);
    BS_PLAIN(K_COLL, k_coll_apply, D, mode);
}
void ghost(const Dev& D, const Launch& L, int precision, int use_mls) {
    BS_DISPATCH(K_GHOST, precision, k_ghost, D, use_mls);
}

}  // namespace bs
