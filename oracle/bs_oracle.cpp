// bs_oracle.cpp -- TEST INFRASTRUCTURE ONLY (parity checker and CPU baseline).
//
// FP64 restatement of the reference's per-step ISPH hot path
// (Sinchanrc/Beach-Slope, Fortran 2008 + OpenMP).  It keeps the reference's
// own data model on purpose -- a grid of cells, each with a particle slot
// list (plist), per-slot properties (pplist), per-slot neighbour lists of
// slot pointers with stored distance and kernel gradient (verlet), and the
// eight-way cell transfer lists -- so that slot order, matid numbering and
// every stale-value semantic of the reference carry over.  Every routine
// cites the reference file:line it restates.
//
// Build: compiled with -O2 -fopenmp -ffp-contract=off (no FMA contraction:
// the pair-distance test must round exactly as written).
#include "bs_oracle.h"

#include <algorithm>
#include <cmath>
#include <cstdint>
#include <cstdio>
#include <cstring>
#include <limits>
#include <string>
#include <vector>
#ifdef _OPENMP
#include <omp.h>
#endif

namespace {

// ---- literal constants with the reference's precision (default REAL is single) ----
const double ALP = 0.1;                          // kernel.f90:30 (real(dp))
const double C28 = (double)(28.0f * 3.14f);      // kernel.f90:61 "28.0*3.14" evaluated in single
const double C3 = (double)(3.0f * 3.14f);        // kernel.f90:62 "3.0*3.14"
const double SP_1EM5 = (double)1e-5f;            // functions.f90:324
const double SP_1EM6 = (double)1e-6f;            // integrator.f90:581, scalar.f90:322
const double SP_1EM9 = (double)1e-9f;            // scalar.f90:246, integrator.f90:892 (Dm)

struct Particle {   // particles, particle.f90:31-47
    double mass = 0, density = 0, pressure = 0, vx = 0, vy = 0, vxs = 0, vys = 0, x = 0, y = 0,
           xs = 0, ys = 0, con = 0, ovol = 0, oden = 0, tden = 0;
    int tid = 0, pid = 0, matid = 0;
    bool free = false, vicinity = false, buffer = false;
};

struct Props {      // properties, particle.f90:60-69 (per SLOT, not per particle)
    double coff[4] = {0, 0, 0, 0};
    double cdiff = 0, gradvx = 0, vel = 0, nut = 0, tke = 0, porosity = 1.0, resistx = 0,
           resisty = 0, varts = 0;
};

struct NbrRef { int cell, slot; };   // list%nh(m)%part => cellX%plist(slot)

struct Verlet {     // verlet, interactions.f90:26-35
    std::vector<NbrRef> nh;
    std::vector<double> dist, kx, ky;   // dist(:), klt(1,:), klt(2,:)
    int count = 0;
};

struct Grain { double x, y, mass, density; };

struct Cell {       // cell, domain.f90:28-46
    std::vector<Particle> plist;
    std::vector<Props> pplist;
    std::vector<Verlet> list;
    std::vector<Grain> porlist;
    std::vector<int> ftemp;
    std::vector<Particle> tr[8];   // tn, ts, tw, te, tse, tne, tsw, tnw
    double xleft = 0, xright = 0, ytop = 0, ybot = 0, maxvel = 0, maxeddy = 0;
    int ptot = 0, btot = 0;
};

enum { TN = 0, TS, TW, TE, TSE, TNE, TSW, TNW };

struct Row {        // matrixsetup, particle.f90:49-53
    int sz = 0;
    std::vector<double> val;
    std::vector<int> col;
    std::vector<double> off_aligned;   // scaled value per neighbour m (export only)
    double diag_total = 0;             // sum of scaled entries with col == row (export only)
};

inline double sq(double a) { return a * a; }

// kernel.f90:34-66 (hybrid: 0.1 cubic spline + 0.9 hyperbolic)
double Wab(double radial, double smln) {
    double t1 = (radial < smln)
                    ? (4.0 - (6.0 * (radial * radial) / (smln * smln)) +
                       (3.0 * (radial * radial * radial) / (smln * smln * smln)))
                    : (2.0 - radial / smln) * (2.0 - radial / smln) * (2.0 - radial / smln);
    double t2 = (radial < smln)
                    ? ((radial / smln) * (radial / smln) * (radial / smln) - (6.0 * radial / smln) + 6.0)
                    : (2.0 - radial / smln) * (2.0 - radial / smln) * (2.0 - radial / smln);
    return ALP * t1 * (10.0 / (C28 * (smln * smln))) + (1.0 - ALP) * t2 * (1.0 / (C3 * (smln * smln)));
}

// kernel.f90:68-92
double Wo(double smln) {
    return ALP * 4.0 * (10.0 / (C28 * (smln * smln))) + (1.0 - ALP) * 6.0 * (1.0 / (C3 * (smln * smln)));
}

// kernel.f90:94-127 / 129-162 (and hWabx/hWaby 204-248, identical): gradient
// w.r.t. p2 for the pair (p1, p2); d = p2 - p1 component ("p2%x-p1%x").
inline double Wgrad(double d21, double radial, double smln) {
    double t1 = (radial < smln)
                    ? ((9.0 * radial / (smln * smln * smln)) - (12.0 / (smln * smln))) * d21
                    : ((3.0 / (radial * smln)) * sq(2.0 - radial / smln)) * (-d21);
    double t2 = (radial < smln)
                    ? ((3.0 * radial / (smln * smln * smln)) - 6.0 / (radial * smln)) * d21
                    : ((3.0 / (radial * smln)) * sq(2.0 - radial / smln)) * (-d21);
    return ALP * t1 * (10.0 / (C28 * (smln * smln))) + (1.0 - ALP) * t2 * (1.0 / (C3 * (smln * smln)));
}
inline double Wabx(const Particle& p1, const Particle& p2, double r, double h) {
    return Wgrad(p2.x - p1.x, r, h);
}
inline double Waby(const Particle& p1, const Particle& p2, double r, double h) {
    return Wgrad(p2.y - p1.y, r, h);
}

// functions.f90:28-42
inline double dist(double x1, double y1, double x2, double y2) {
    return std::sqrt(((x1 - x2) * (x1 - x2)) + ((y1 - y2) * (y1 - y2)));
}

// functions.f90:62-96
void invertmat2D(double a[4]) {
    double arr11 = a[3], arr12 = -a[1], arr21 = -a[2], arr22 = a[0];
    double det = a[0] * a[3] - a[1] * a[2];
    if (std::fabs(det) >= SP_1EM5 && !std::isnan(det) && std::isfinite(det)) {
        a[0] = arr11 / det; a[1] = arr12 / det; a[2] = arr21 / det; a[3] = arr22 / det;
    } else {
        a[0] = 1.0; a[1] = 0.0; a[2] = 0.0; a[3] = 1.0;
    }
}

// integrator.f90:12-30 (= porous.f90:12-30)
inline double vis(double oden) {
    double Sp = oden - 1000.0;
    const double Acn = 0.001652, Bcn = 0.0000083;
    return (1.002 + Acn * Sp + Bcn * (Sp * Sp)) * 0.001;
}

}  // namespace

struct OrZone {      // one open-boundary buffer zone (buffer1 / buffer2 + entrycell1 / 2)
    bool set = false;
    std::vector<Particle> tmpl;
    std::vector<std::pair<int, int>> cells;
    double period = 0, phase = 0, remove_x = 0;
    int side = 1;
    long next_k = 1;
};

struct or_scene {
    bs_params P;
    OrZone zones[2];
    int cellx, celly;
    double h, lam, dl, cw;
    std::vector<Cell> cells;
    double t = 0, dt = 0, dtsol = 0, umax = 0, numax = 0;
    int solsteps = 1;
    std::vector<Row> rows;
    std::vector<double> fvec, fsol;
    int nrows = 0;
    bool assembled = false;
    int last_iters = 0, last_outer = 0;
    double last_relres = 0;
    unsigned err = 0;

    Cell& C(int i, int j) { return cells[(size_t)(j - 1) * celly + (i - 1)]; }
    int key(int i, int j) const { return (j - 1) * celly + (i - 1); }
};

namespace {

// setup.f90:120-123
double xleft_of(const or_scene* s, int j) { return (double)(j - 2) * (4.0 * s->h); }
double xright_of(const or_scene* s, int j) { return (double)(j - 1) * (4.0 * s->h); }
double ybot_of(const or_scene* s, int i) { return (double)(-i + s->celly - 1) * (4.0 * s->h); }
double ytop_of(const or_scene* s, int i) { return (double)(-i + s->celly) * (4.0 * s->h); }

bool locate(const or_scene* s, double x, double y, int* ci, int* cj) {
    if (!std::isfinite(x) || !std::isfinite(y)) return false;
    int j = (int)std::floor(x / s->cw) + 2;
    j = std::max(1, std::min(s->cellx, j));
    for (int it = 0; it < 4; ++it) {
        if (x < xleft_of(s, j) && j > 1) --j;
        else if (!(x < xright_of(s, j)) && j < s->cellx) ++j;
        else break;
    }
    int i = s->celly - 1 - (int)std::floor(y / s->cw);
    i = std::max(1, std::min(s->celly, i));
    for (int it = 0; it < 4; ++it) {
        if (y < ybot_of(s, i) && i < s->celly) ++i;
        else if (!(y < ytop_of(s, i)) && i > 1) --i;
        else break;
    }
    if (!(x >= xleft_of(s, j) && x < xright_of(s, j) && y >= ybot_of(s, i) && y < ytop_of(s, i)))
        return false;
    if (i < 2 || i > s->celly - 1 || j < 2 || j > s->cellx - 1) return false;
    *ci = i; *cj = j;
    return true;
}

void ensure_slots(Cell& c) {
    if ((int)c.pplist.size() < c.ptot) c.pplist.resize(c.ptot);
    if ((int)c.list.size() < c.ptot) c.list.resize(c.ptot);
}

// Quadrant of a particle within its cell: search.f90:328-388 (the fifth,
// equality, branch is unreachable after the first one).
// Returns the four cells in the reference's order cell1..cell4.
bool quadrant(const or_scene* s, const Cell& c, const Particle& p, int i, int j, int out[4][2]) {
    double mx = c.xleft + std::fabs((c.xleft - c.xright) / 2.0);
    double my = c.ybot + std::fabs((c.ytop - c.ybot) / 2.0);
    (void)s;
    if (p.x <= mx && p.y <= my) {
        int o[4][2] = {{i, j - 1}, {i + 1, j - 1}, {i, j}, {i + 1, j}};
        std::memcpy(out, o, sizeof(o));
    } else if (p.x > mx && p.y <= my) {
        int o[4][2] = {{i, j}, {i + 1, j}, {i, j + 1}, {i + 1, j + 1}};
        std::memcpy(out, o, sizeof(o));
    } else if (p.x > mx && p.y > my) {
        int o[4][2] = {{i - 1, j}, {i, j}, {i - 1, j + 1}, {i, j + 1}};
        std::memcpy(out, o, sizeof(o));
    } else if (p.x <= mx && p.y > my) {
        int o[4][2] = {{i - 1, j - 1}, {i, j - 1}, {i - 1, j}, {i, j}};
        std::memcpy(out, o, sizeof(o));
    } else {
        return false;   // NaN position: the reference keeps stale cell pointers
    }
    return true;
}

template <class F>
void for_interior(or_scene* s, F f) {
    const int nx = s->cellx - 2, ny = s->celly - 2;
    const long tot = (long)nx * ny;
#pragma omp parallel for schedule(dynamic, 16)
    for (long q = 0; q < tot; ++q) {
        int j = 2 + (int)(q / ny), i = 2 + (int)(q % ny);
        f(i, j);
    }
}

// ---------------------------------------------------------------- projection
// isph.f90:17-47
void projection(or_scene* s) {
    for_interior(s, [&](int i, int j) {
        Cell& c = s->C(i, j);
        for (int k = 0; k < c.ptot; ++k) {
            Particle& p = c.plist[k];
            if (p.tid == 3) {
                const double por = c.pplist[k].porosity;
                p.xs = p.x;
                p.x = p.x + (s->dt * p.vx / por);
                p.ys = p.y;
                p.y = p.y + (s->dt * p.vy / por);
            }
        }
    });
}

// ------------------------------------------------------ cellshift / cellshiftalt
// integrator.f90:251-392 (alt=false) and 33-249 (alt=true: outflow cut-offs 61-62)
void cellshift(or_scene* s, bool alt) {
    const double xlc = s->P.xlcutoff, ytc = s->P.ytcutoff;
    for_interior(s, [&](int i, int j) {
        Cell& c = s->C(i, j);
        c.ftemp.clear();
        for (auto& t : c.tr) t.clear();
        for (int k = 0; k < c.ptot; ++k) {   // "must be carried out serially"
            const Particle& p = c.plist[k];
            if (p.tid != 3) continue;
            const double x1 = p.x, y1 = p.y;
            const bool keep = !alt || (x1 > xlc) || p.buffer || ((x1 <= xlc) && (y1 <= ytc));
            int d = -2;   // -1 stay, -2 lost
            if ((x1 >= c.xleft) && (x1 < c.xright)) {
                if ((y1 >= c.ybot) && (y1 < c.ytop)) d = -1;
                else if (y1 < c.ybot) d = TS;
                else if (y1 >= c.ytop) d = TN;
            } else if (x1 >= c.xright) {
                if (y1 >= c.ytop) d = TNE;
                else if ((y1 >= c.ybot) && (y1 < c.ytop)) d = TE;
                else if (y1 < c.ybot) d = TSE;
            } else if (x1 < c.xleft) {
                if (y1 >= c.ytop) d = TNW;
                else if ((y1 >= c.ybot) && (y1 < c.ytop)) d = TW;
                else if (y1 < c.ybot) d = TSW;
            }
            if (!keep || d == -2) continue;
            if (d == -1) c.ftemp.push_back(k);
            else c.tr[d].push_back(p);
        }
    });
    // particle transfers (integrator.f90:319-390), into a fresh list per cell
    std::vector<std::vector<Particle>> newlist((size_t)s->cellx * s->celly);
    for_interior(s, [&](int i, int j) {
        Cell& c = s->C(i, j);
        auto& nl = newlist[s->key(i, j)];
        nl.reserve(c.ptot + 8);
        for (int k = 0; k < c.btot; ++k) nl.push_back(c.plist[k]);
        for (int k : c.ftemp) nl.push_back(c.plist[k]);
        auto take = [&](int ii, int jj, int d) {
            for (const auto& p : s->C(ii, jj).tr[d]) nl.push_back(p);
        };
        take(i + 1, j, TN);
        take(i - 1, j, TS);
        take(i, j + 1, TW);
        take(i, j - 1, TE);
        take(i - 1, j - 1, TSE);
        take(i + 1, j - 1, TNE);
        take(i - 1, j + 1, TSW);
        take(i + 1, j + 1, TNW);
    });
    // particles sent to a border cell are lost (the gather loop never runs there)
    long before = 0, after = 0;
    for (int j = 2; j <= s->cellx - 1; ++j)
        for (int i = 2; i <= s->celly - 1; ++i) {
            Cell& c = s->C(i, j);
            before += c.ptot;
            c.plist.swap(newlist[s->key(i, j)]);
            c.ptot = (int)c.plist.size();
            after += c.ptot;
            ensure_slots(c);
        }
    if (after < before && !alt) s->err |= BS_ERR_LOST_PARTICLE;
    for (int j = 2; j <= s->cellx - 1; ++j)
        for (int i = 2; i <= s->celly - 1; ++i)
            for (auto& t : s->C(i, j).tr) t.clear();
}

// isph.f90:88-113
void resetid(or_scene* s) {
    int mat_count = 0;
    for (int j = 1; j <= s->cellx; ++j)
        for (int i = 1; i <= s->celly; ++i) {
            Cell& c = s->C(i, j);
            for (int k = 0; k < c.ptot; ++k) c.plist[k].matid = ++mat_count;
        }
}

// ------------------------------------------------------------------ search
// nsearch2, search.f90:13-308
void nsearch2(or_scene* s, int ci, int cj, int n, int cells4[4][2]) {
    Cell& cn = s->C(ci, cj);
    Particle& p = cn.plist[n];
    Props& pp = cn.pplist[n];
    Verlet& L = cn.list[n];
    const double smln = s->h;
    L.count = 0;
    L.nh.clear(); L.dist.clear(); L.kx.clear(); L.ky.clear();
    double res[4] = {0, 0, 0, 0};
    p.free = false;
    pp.gradvx = 0.0;
    for (int q = 0; q < 4; ++q) {
        const int ii = cells4[q][0], jj = cells4[q][1];
        const Cell& c = s->C(ii, jj);
        const int ck = s->key(ii, jj);
        for (int c2 = 0; c2 < c.ptot; ++c2) {
            const Particle& o = c.plist[c2];
            if ((p.tid != o.tid) || ((p.tid == o.tid) && (p.matid != o.matid))) {
                const double radial = dist(p.x, p.y, o.x, o.y);
                if (radial < (2.0 * smln)) {
                    L.count += 1;
                    L.nh.push_back({ck, c2});
                    L.dist.push_back(radial);
                    const double res2 = Wabx(o, p, radial, smln);
                    const double res4 = Waby(o, p, radial, smln);
                    L.kx.push_back(res2);
                    L.ky.push_back(res4);
                    const double res1 = (o.mass) * (o.x - p.x) / (o.density);
                    const double res3 = (o.mass) * (o.y - p.y) / (o.density);
                    res[0] = res[0] + res2 * res1;
                    res[1] = res[1] + res4 * res1;
                    res[2] = res[2] + res2 * res3;
                    res[3] = res[3] + res4 * res3;
                }
            }
        }
    }
    if (p.tid == 3) {
        p.free = false;
        p.vicinity = false;
        pp.gradvx = (res[0] + res[3]);
        invertmat2D(res);
        for (int q = 0; q < 4; ++q) pp.coff[q] = res[q];
        if ((pp.gradvx <= (s->P.lamfs * s->P.maxdivr)) && !p.buffer) p.free = true;
    }
}

// neighbour, search.f90:310-399
void neighbour(or_scene* s) {
    for_interior(s, [&](int i, int j) {
        Cell& c = s->C(i, j);
        ensure_slots(c);
        for (int k = 0; k < c.ptot; ++k) {
            int cells4[4][2];
            if (!quadrant(s, c, c.plist[k], i, j, cells4)) {
                c.list[k].count = 0;
                c.list[k].nh.clear(); c.list[k].dist.clear(); c.list[k].kx.clear(); c.list[k].ky.clear();
                continue;
            }
            nsearch2(s, i, j, k, cells4);
        }
    });
}

// ------------------------------------------------------------------ porosity
// effpor + porsearch, porous.f90:32-224
void effpor(or_scene* s, bool keep_density = false) {
    const double por = s->P.por, lamk = s->P.lamk, d50 = s->P.d50, h1 = s->h;
    for_interior(s, [&](int i, int j) {
        Cell& c = s->C(i, j);
        ensure_slots(c);
        for (int k = 0; k < c.ptot; ++k) {
            Particle& p = c.plist[k];
            Props& pp = c.pplist[k];
            double solidfrac = 0.0;
            pp.resistx = 0.0;
            pp.resisty = 0.0;
            if (p.tid != 3) continue;
            pp.porosity = 1.0;
            const double mx = c.xleft + std::fabs((c.xleft - c.xright) / 2.0);
            const double my = c.ybot + std::fabs((c.ytop - c.ybot) / 2.0);
            int cs[4][2] = {{i, j}, {i, j}, {i, j}, {i, j}};
            if (p.x <= mx && p.y <= my) {
                int o[3][2] = {{i, j - 1}, {i + 1, j}, {i + 1, j - 1}};
                std::memcpy(cs + 1, o, sizeof(o));
            } else if (p.x > mx && p.y <= my) {
                int o[3][2] = {{i, j + 1}, {i + 1, j}, {i + 1, j + 1}};
                std::memcpy(cs + 1, o, sizeof(o));
            } else if (p.x > mx && p.y > my) {
                int o[3][2] = {{i - 1, j + 1}, {i - 1, j}, {i, j + 1}};
                std::memcpy(cs + 1, o, sizeof(o));
            } else if (p.x <= mx && p.y > my) {
                int o[3][2] = {{i - 1, j}, {i - 1, j - 1}, {i, j - 1}};
                std::memcpy(cs + 1, o, sizeof(o));
            }
            for (int q = 0; q < 4; ++q) {   // porsearch, porous.f90:48-103
                const Cell& g = s->C(cs[q][0], cs[q][1]);
                for (const Grain& gr : g.porlist) {
                    const double radial = dist(p.x, p.y, gr.x, gr.y);
                    if (radial < (2.0 * h1))
                        solidfrac = solidfrac + (1.0 - por * 1.0) * Wab(radial, h1) * gr.mass / gr.density;
                }
            }
            if (solidfrac > (1.0 - por)) solidfrac = 1.0 - por;
            pp.porosity = 1.0 - solidfrac;
            if (!keep_density) p.density = pp.porosity * p.oden;   // WCSPH keeps its own density
            const double phi = pp.porosity;
            const double Fch = 1.750 / (std::sqrt(150 * (phi * phi * phi)));
            const double vmag = std::sqrt(p.vx * p.vx + p.vy * p.vy);
            const double r = -((vis(p.oden) / p.oden) * lamk * ((1.0 - phi) * (1.0 - phi)) /
                               ((phi * phi * phi) * (d50 * d50))) -
                             ((Fch * vmag * std::sqrt(lamk) * (1.0 - phi)) /
                              (std::sqrt(phi * phi * phi) * d50));
            pp.resistx = r;
            pp.resisty = r;
        }
    });
}

// --------------------------------------------------------------- eddyvis
// turbulence.f90:12-113
void eddyvis(or_scene* s) {
    const double cv = 0.080, ce = 1.0, cs = 0.150, dl = s->dl;
    for_interior(s, [&](int i, int j) {
        Cell& c = s->C(i, j);
        for (int k = c.btot; k < c.ptot; ++k) {
            const Particle& p = c.plist[k];
            Props& pp = c.pplist[k];
            const Verlet& L = c.list[k];
            double t1 = 0, t2 = 0, t3 = 0;
            for (int m = 0; m < L.count; ++m) {
                const Cell& oc = s->cells[L.nh[m].cell];
                const Particle& x = oc.plist[L.nh[m].slot];
                const Props& y = oc.pplist[L.nh[m].slot];
                const double z1 = L.kx[m], z2 = L.ky[m];
                t1 = t1 + (x.mass * (x.vx / y.porosity - p.vx / pp.porosity) *
                           (pp.coff[0] * z1 + pp.coff[1] * z2)) / x.density;
                t2 = t2 + (x.mass * (x.vy / y.porosity - p.vy / pp.porosity) *
                           (pp.coff[2] * z1 + pp.coff[3] * z2)) / x.density;
                t3 = t3 + (0.50 * x.mass *
                           ((x.vx / y.porosity - p.vx / pp.porosity) * (pp.coff[2] * z1 + pp.coff[3] * z2) +
                            (x.vy / y.porosity - p.vy / pp.porosity) * (pp.coff[0] * z1 + pp.coff[1] * z2))) /
                              x.density;
            }
            const double t4 = std::sqrt(2 * (t1 * t1 + t2 * t2) + (2 * t3) * (2 * t3));
            pp.nut = ((cs * dl) * (cs * dl)) * t4;
            pp.tke = (cv / ce) * ((dl * t4) * (dl * t4));
        }
    });
}

// --------------------------------------------------------------- int_vel
// integrator.f90:459-703
void int_vel(or_scene* s) {
    const double dl = s->dl, dt = s->dt, g = s->P.g, lam = s->lam, h1 = s->h, umax = s->umax;
    const double ps = 1.0;
    for_interior(s, [&](int i, int j) {   // varts for free particles (468-507)
        Cell& c = s->C(i, j);
        for (int k = 0; k < c.ptot; ++k) {
            const Particle& p = c.plist[k];
            Props& pp = c.pplist[k];
            if (!p.free) continue;
            double t1 = 0, t2 = 0;
            pp.varts = 0.0;
            const Verlet& L = c.list[k];
            for (int m = 0; m < L.count; ++m) {
                const Cell& oc = s->cells[L.nh[m].cell];
                const Particle& x = oc.plist[L.nh[m].slot];
                const Props& y = oc.pplist[L.nh[m].slot];
                const double z1 = L.kx[m], z2 = L.ky[m];
                t1 = t1 + (x.vx / y.porosity - p.vx / pp.porosity) * (pp.coff[0] * z1 + pp.coff[1] * z2) *
                              (x.mass / x.density);
                t2 = t2 + (x.vy / y.porosity - p.vy / pp.porosity) * (pp.coff[2] * z1 + pp.coff[3] * z2) *
                              (x.mass / x.density);
            }
            pp.varts = ps * (dl * dl) * std::sqrt(t1 * t1 + t2 * t2) * std::sqrt(p.vx * p.vx + p.vy * p.vy) /
                       ((umax + SP_1EM6) * pp.porosity);
        }
    });
    const double wo = Wo(h1);
    for_interior(s, [&](int i, int j) {   // non-pressure velocity (510-701)
        Cell& c = s->C(i, j);
        for (int k = 0; k < c.ptot; ++k) {
            Particle& p = c.plist[k];
            const Props& pp = c.pplist[k];
            const Verlet& L = c.list[k];
            if ((p.tid == 3) && !p.buffer) {
                p.vxs = 0.0;
                p.vys = 0.0;
                for (int m = 0; m < L.count; ++m) {
                    const Cell& oc = s->cells[L.nh[m].cell];
                    const Particle& x = oc.plist[L.nh[m].slot];
                    const Props& y = oc.pplist[L.nh[m].slot];
                    const double z1 = L.kx[m], z2 = L.ky[m];
                    double cmu;
                    if (x.tid == 3) {
                        cmu = 2 * vis(p.oden) * vis(x.oden) * ((1.0 / p.oden) * (1.0 / x.oden)) /
                              ((vis(p.oden) / p.oden) + (vis(x.oden) / x.oden));
                    } else {
                        cmu = vis(p.oden) * (1.0 / p.oden);
                    }
                    double vart;
                    if (p.free) vart = pp.varts;
                    else if (!p.free && x.free && !p.buffer) vart = Wab(L.dist[m], h1) * y.varts / wo;
                    else vart = 0.0;
                    const double pvol = x.mass / x.density;
                    const double p_dist = 1.0 / (L.dist[m] * L.dist[m] + lam);
                    double t1 = (2 * pvol * (p.vx - x.vx) * (p.x - x.x) * (pp.coff[0] * z1 + pp.coff[1] * z2)) * p_dist;
                    double t2 = (2 * pvol * (p.vx - x.vx) * (p.y - x.y) * (pp.coff[2] * z1 + pp.coff[3] * z2)) * p_dist;
                    p.vxs = p.vxs + (t1 + t2) * (cmu + vart);
                    if (x.tid > 2) {
                        if ((pp.nut < SP_1EM6) && (y.nut < SP_1EM6))
                            p.vxs = p.vxs + (t1 + t2) * (pp.nut + y.nut) * 0.50;
                        else
                            p.vxs = p.vxs + (t1 + t2) * ((2 * pp.nut * y.nut) / (pp.nut + y.nut));
                    }
                    t1 = (2 * pvol * (p.vy - x.vy) * (p.x - x.x) * (pp.coff[0] * z1 + pp.coff[1] * z2)) * p_dist;
                    t2 = (2 * pvol * (p.vy - x.vy) * (p.y - x.y) * (pp.coff[2] * z1 + pp.coff[3] * z2)) * p_dist;
                    p.vys = p.vys + (t1 + t2) * (cmu + vart);
                    if (x.tid > 2) {
                        if ((pp.nut < SP_1EM6) && (y.nut < SP_1EM6))
                            p.vys = p.vys + (t1 + t2) * (pp.nut + y.nut) * 0.50;
                        else
                            p.vys = p.vys + (t1 + t2) * ((2 * pp.nut * y.nut) / (pp.nut + y.nut));
                    }
                    if (p.tid == 3) {   // turbulence (644-665)
                        t1 = (pvol * (y.tke - pp.tke) * (pp.coff[0] * z1 + pp.coff[1] * z2));
                        p.vxs = p.vxs - (t1)*pp.porosity * 2.0 / 3;
                        t1 = (pvol * (y.tke - pp.tke) * (pp.coff[2] * z1 + pp.coff[3] * z2));
                        p.vys = p.vys - (t1)*pp.porosity * 2.0 / 3;
                    }
                }
                p.vxs = (p.vx + (dt * p.vxs)) / (1.0 - dt * pp.resistx * pp.porosity);
                p.vys = (p.vy + dt * (p.vys)) / (1.0 - dt * pp.resisty * pp.porosity);
                p.vys = p.vys + g * pp.porosity * dt;
            }
            if (p.buffer) {
                p.vxs = p.vx;
                p.vys = g * pp.porosity * dt;
            }
        }
    });
}

// ------------------------------------------------------------ PPE assembly
// ppesolve, isph.f90:115-456 (+ sort, qsort.f90:57-88)
int count_particles(or_scene* s) {
    int n = 0;
    for (auto& c : s->cells) n += c.ptot;
    return n;
}

void ppe_assemble(or_scene* s) {
    const int n = count_particles(s);
    s->nrows = n;
    s->rows.assign(n, Row());
    s->fvec.assign(n, 0.0);
    const double dt = s->dt, lam = s->lam, rho = s->P.rho, rel_den = s->P.rel_den;
    for_interior(s, [&](int i, int j) {
        Cell& c = s->C(i, j);
        for (int k = 0; k < c.ptot; ++k) {
            const Particle& p = c.plist[k];
            const Props& pp = c.pplist[k];
            const Verlet& L = c.list[k];
            const int pos = p.matid;     // 1-based row
            const int num = L.count;
            Row& R = s->rows[pos - 1];
            // row initialisation (isph.f90:123-131): val=0, val(1)=1, col=row
            const int width = num + 1;
            R.val.assign(width, 0.0);
            R.val[0] = 1.0;
            R.col.assign(width, pos);
            R.off_aligned.assign(num, 0.0);
            std::vector<int> ins_of(num, -1);
            int dia_pt = 1, ins_pt = 0;
            double dia_term = 0.0;
            R.sz = num + 1;
            double fv = 0.0;
            const double rho_i = p.density * (1.0 / pp.porosity);
            for (int m = 1; m <= num; ++m) {
                const Cell& oc = s->cells[L.nh[m - 1].cell];
                const Particle& x = oc.plist[L.nh[m - 1].slot];
                const Props& y = oc.pplist[L.nh[m - 1].slot];
                const double z1 = L.kx[m - 1], z2 = L.ky[m - 1];
                if (pos > x.matid) { dia_pt = m + 1; ins_pt = m; }
                else ins_pt = m + 1;
                double lamp;
                if (p.free && (x.tid == 3)) lamp = (1.0 + x.oden / (rho * rel_den));
                else lamp = 1.0;
                const double rho_j = x.density * (1.0 / y.porosity);
                const double pvol = x.mass * (1.0 / x.density);
                const double r = dist(x.x, x.y, p.x, p.y);
                const double p_dist = 1.0 / ((r * r) + lam);
                const double rho_ij = 2 * x.density * p.density * (1.0 / ((y.porosity) * (pp.porosity))) *
                                      (1.0 / ((x.density * (1.0 / y.porosity)) + (p.density * (1.0 / pp.porosity))));
                double t1, t2;
                if (p.tid == 3) {
                    t1 = 2 * pvol * ((pp.coff[0] * z1 + pp.coff[1] * z2)) * (p.x - x.x) * (p_dist);
                    t2 = 2 * pvol * ((pp.coff[2] * z1 + pp.coff[3] * z2)) * (p.y - x.y) * (p_dist);
                    R.val[ins_pt - 1] = (-(t1 + t2));
                    R.col[ins_pt - 1] = x.matid;
                    ins_of[m - 1] = ins_pt;
                    dia_term = dia_term + (t1 + t2) * lamp;
                    if (x.tid == 3) {
                        t1 = (pvol * (x.vxs * rho_ij / y.porosity - p.vxs * rho_ij / pp.porosity) *
                              (pp.coff[0] * z1 + pp.coff[1] * z2));
                        t2 = (pvol * (x.vys * rho_ij / y.porosity - p.vys * rho_ij / pp.porosity) *
                              (pp.coff[2] * z1 + pp.coff[3] * z2));
                    } else {
                        t1 = (pvol * (x.vxs * rho_i / pp.porosity - p.vxs * rho_i / pp.porosity) *
                              (pp.coff[0] * z1 + pp.coff[1] * z2));
                        t2 = (pvol * (x.vys * rho_i / pp.porosity - p.vys * rho_i / pp.porosity) *
                              (pp.coff[2] * z1 + pp.coff[3] * z2));
                    }
                    fv = fv + (t1 + t2) / dt;
                } else if (p.tid == 2) {
                    t1 = 2 * pvol * (z1) * (p.x - x.x) * (p_dist);
                    t2 = 2 * pvol * (z2) * (p.y - x.y) * (p_dist);
                    if (x.tid <= 2) {
                        R.val[ins_pt - 1] = -(t1 + t2);
                        R.col[ins_pt - 1] = x.matid;
                        ins_of[m - 1] = ins_pt;
                        dia_term = dia_term + (t1 + t2);
                    }
                } else if (p.tid == 1) {
                    if (x.tid == 3) {
                        t1 = 2 * p.mass * ((y.coff[0] * z1 + y.coff[1] * z2)) * (p.x - x.x) * (p_dist) / ((p.density));
                        t2 = 2 * p.mass * ((y.coff[2] * z1 + y.coff[3] * z2)) * (p.y - x.y) * (p_dist) / ((p.density));
                        R.val[ins_pt - 1] = -(t1 + t2);
                        R.col[ins_pt - 1] = x.matid;
                        ins_of[m - 1] = ins_pt;
                        dia_term = dia_term + (t1 + t2);
                        t1 = (p.mass * (x.vxs * rho_j / y.porosity - p.vxs * rho_j / pp.porosity) *
                              (y.coff[0] * z1 + y.coff[1] * z2)) / (p.density);
                        t2 = (p.mass * (x.vys * rho_j / y.porosity - p.vys * rho_j / pp.porosity) *
                              (y.coff[2] * z1 + y.coff[3] * z2)) / (p.density);
                        fv = fv + (t1 + t2) / dt;
                    } else if (x.tid <= 2) {
                        t1 = 2 * pvol * (z1) * (p.x - x.x) * (p_dist);
                        t2 = 2 * pvol * (z2) * (p.y - x.y) * (p_dist);
                        R.val[ins_pt - 1] = -(t1 + t2);
                        R.col[ins_pt - 1] = x.matid;
                        ins_of[m - 1] = ins_pt;
                        dia_term = dia_term + (t1 + t2);
                    }
                }
            }
            R.val[dia_pt - 1] = dia_term;
            R.col[dia_pt - 1] = pos;
            const double t1 = R.val[dia_pt - 1];
            fv = fv / t1;   // Jacobi scaling (isph.f90:436-440)
            for (int m = 0; m < width; ++m) R.val[m] = R.val[m] / t1;
            // aligned export: entries written by a neighbour, and everything at col==row
            R.diag_total = 0.0;
            std::vector<char> used(width, 0);
            for (int m = 0; m < num; ++m)
                if (ins_of[m] > 0 && ins_of[m] != dia_pt) {
                    // a later neighbour may have reused the slot only if ins_pt repeats; it does not
                    R.off_aligned[m] = R.val[ins_of[m] - 1];
                    used[ins_of[m] - 1] = 1;
                }
            for (int q = 0; q < width; ++q)
                if (!used[q] && R.col[q] == pos) R.diag_total += R.val[q];
            if (num > 0) {   // sort by column (qsort.f90:57-88); stable for the col==row duplicates
                std::vector<int> ord(width);
                for (int q = 0; q < width; ++q) ord[q] = q;
                std::stable_sort(ord.begin(), ord.end(), [&](int a, int b) { return R.col[a] < R.col[b]; });
                std::vector<double> v2(width);
                std::vector<int> c2(width);
                for (int q = 0; q < width; ++q) { v2[q] = R.val[ord[q]]; c2[q] = R.col[ord[q]]; }
                R.val.swap(v2);
                R.col.swap(c2);
            }
            s->fvec[pos - 1] = fv;
            if (!(dia_term != 0.0)) {
#pragma omp atomic
                s->err |= BS_ERR_ZERO_DIAG;
            }
        }
    });
    s->assembled = true;
}

// spmv2, solver.f90:84-127
void spmv2(const or_scene* s, const std::vector<double>& b, std::vector<double>& res) {
    const int n = s->nrows;
#pragma omp parallel for schedule(static)
    for (int is = 0; is < n; ++is) {
        const Row& R = s->rows[is];
        double sol = 0.0;
        for (int js = 0; js < R.sz; ++js) sol = sol + R.val[js] * b[R.col[js] - 1];
        res[is] = sol;
    }
}

// vecvec, solver.f90:8-25.  Each thread sums a fixed contiguous range and the
// partial sums are added in thread order, so the result depends only on the
// thread count (an OpenMP reduction clause combines in arrival order); on one
// thread it is the sequential sum.
double vecvec(const std::vector<double>& a, const std::vector<double>& b) {
    const long n = (long)a.size();
    std::vector<double> part(omp_get_max_threads(), 0.0);
#pragma omp parallel
    {
        const int t = omp_get_thread_num(), nt = omp_get_num_threads();
        const long lo = n * t / nt, hi = n * (t + 1) / nt;
        double s = 0.0;
        for (long k = lo; k < hi; ++k) s = s + a[k] * b[k];
        part[t] = s;
    }
    double res = 0.0;
    for (double v : part) res = res + v;
    return res;
}

// bicgstab, solver.f90:129-254, generic over the operator.  rule 0 stops on
// the recurrence residual ||rs||/||b|| <= tol (then reports the true one);
// rule 1 is the reference's relative-change rule (233-242).
template <class Op>
int bicgstab(int n, Op spmv, const std::vector<double>& b, std::vector<double>& sl, double tol, int maxit,
             int rule, int* iters, double* relres) {
    std::vector<double> guess(sl), rs(n), p(n), res(n), mm1(n), mm2(n), si(n);
    const double itls = (double)1e-2f;
    spmv(guess, res);
    for (int k = 0; k < n; ++k) { rs[k] = b[k] - res[k]; p[k] = rs[k]; res[k] = rs[k]; }
    const double bnorm = std::sqrt(vecvec(b, b));
    int it = 0, status = 0;
    double rn = std::sqrt(vecvec(rs, rs));
    if (rule == 0 && (bnorm == 0.0 || rn / bnorm <= tol)) {
        *iters = 0;
        *relres = bnorm > 0 ? rn / bnorm : 0.0;
        return 0;
    }
    while (true) {
        it++;
        spmv(p, mm1);
        const double prevr = vecvec(res, rs);
        const double alpha = prevr / vecvec(mm1, res);
#pragma omp parallel for schedule(static)
        for (int k = 0; k < n; ++k) si[k] = rs[k] - alpha * mm1[k];
        spmv(si, mm2);
        const double tt = vecvec(mm2, mm2);
        const double wi = (tt != 0.0) ? vecvec(mm2, si) / tt : 0.0;
#pragma omp parallel for schedule(static)
        for (int k = 0; k < n; ++k) {
            sl[k] = sl[k] + alpha * p[k] + wi * si[k];
            rs[k] = si[k] - wi * mm2[k];
        }
        const double betas = (vecvec(rs, res) / prevr) * (alpha / wi);
#pragma omp parallel for schedule(static)
        for (int k = 0; k < n; ++k) p[k] = rs[k] + betas * (p[k] - wi * mm1[k]);
        bool done;
        if (rule == 1) {
            done = true;
            for (int k = 0; k < n; ++k)
                if (std::fabs((sl[k] - guess[k]) / (guess[k] + SP_1EM5)) > itls) {
                    done = false;
                    guess = sl;
                    break;
                }
        } else {
            rn = std::sqrt(vecvec(rs, rs));
            done = (rn / bnorm <= tol) || tt == 0.0 || !std::isfinite(rn);
        }
        if (done) break;
        if (it >= maxit) { status = 1; break; }
    }
    // true residual
    spmv(sl, res);
    double rr = 0.0;
    for (int k = 0; k < n; ++k) rr += (b[k] - res[k]) * (b[k] - res[k]);
    *iters = it;
    *relres = bnorm > 0 ? std::sqrt(rr) / bnorm : std::sqrt(rr);
    return status;
}

// fgmres, solver.f90:306-350: the reference hands the system to MKL's RCI
// dfgmres (Intel oneMKL, closed and absent; no preconditioner, ipar(11) = 0)
// with the relative tolerance dpar(1) on the residual over the initial
// residual (ipar(9) = 1), the zero-norm check of the new Krylov vector
// (ipar(12) = 1, threshold dpar(8) = 1e-12) and the default restart / maximum
// of 150 columns.  Restated from the published algorithm: restarted GMRES
// (Saad & Schultz 1986; flexible form Saad 1993, identical without a
// preconditioner), Arnoldi by modified Gram-Schmidt, Givens rotations on
// the Hessenberg matrix.  rule 0: ||r|| <= tol ||b||; otherwise ||r|| <= tol
// ||r0||.  Returns 1 when maxit columns ran out first.
template <class Op>
int fgmres(int n, Op spmv, const std::vector<double>& b, std::vector<double>& x, double tol, int maxit, int m,
           int rule, int* iters, double* relres) {
    std::vector<double> r(n), w(n);
    std::vector<std::vector<double>> V(m + 1, std::vector<double>(n));
    std::vector<double> H((size_t)(m + 1) * m), cs(m), sn(m), g(m + 1), y(m);
    auto h = [&](int i, int j) -> double& { return H[(size_t)j * (m + 1) + i]; };
    auto residual = [&]() {
        spmv(x, w);
        for (int k = 0; k < n; ++k) r[k] = b[k] - w[k];
        return std::sqrt(vecvec(r, r));
    };
    const double bnorm = std::sqrt(vecvec(b, b));
    double beta = residual();
    const double ref = tol * (rule == 0 ? bnorm : beta);
    int it = 0, status = 0;
    bool conv = bnorm == 0.0 || beta <= ref;
    while (!conv && status == 0) {
        for (int k = 0; k < n; ++k) V[0][k] = r[k] / beta;
        std::fill(g.begin(), g.end(), 0.0);
        g[0] = beta;
        int kcol = 0;
        for (int j = 0; j < m; ++j) {
            spmv(V[j], w);
            for (int i = 0; i <= j; ++i) {
                h(i, j) = vecvec(w, V[i]);
                for (int k = 0; k < n; ++k) w[k] -= h(i, j) * V[i][k];
            }
            const double hn = std::sqrt(vecvec(w, w));
            for (int i = 0; i < j; ++i) {
                const double a = h(i, j), c = h(i + 1, j);
                h(i, j) = cs[i] * a + sn[i] * c;
                h(i + 1, j) = -sn[i] * a + cs[i] * c;
            }
            const double a = h(j, j), den = std::sqrt(a * a + hn * hn);
            cs[j] = den > 0.0 ? a / den : 1.0;
            sn[j] = den > 0.0 ? hn / den : 0.0;
            h(j, j) = den;
            g[j + 1] = -sn[j] * g[j];
            g[j] = cs[j] * g[j];
            ++it;
            kcol = j + 1;
            const double res = std::fabs(g[j + 1]);
            if (!std::isfinite(res)) { status = 1; break; }
            if (res <= ref || hn <= 1e-12) { conv = true; break; }
            if (it >= maxit) { status = 1; break; }
            if (j + 1 < m)
                for (int k = 0; k < n; ++k) V[j + 1][k] = w[k] / hn;
        }
        for (int i = kcol - 1; i >= 0; --i) {
            double acc = 0.0;
            for (int l = i + 1; l < kcol; ++l) acc += h(i, l) * y[l];
            y[i] = h(i, i) != 0.0 ? (g[i] - acc) / h(i, i) : 0.0;
        }
        for (int i = 0; i < kcol; ++i)
            for (int k = 0; k < n; ++k) x[k] += y[i] * V[i][k];
        if (conv || status) break;
        beta = residual();
        conv = beta <= ref;
        if (!std::isfinite(beta)) status = 1;
    }
    const double rt = residual();
    *iters = it;
    *relres = bnorm > 0 ? rt / bnorm : rt;
    return status;
}

int ppe_solve(or_scene* s, double tol, int maxit, int rule, int* iters, double* relres) {
    const int n = s->nrows;
    // warm start: each particle's current pressure at its row
    s->fsol.assign(n, 0.0);
    for (auto& c : s->cells)
        for (int k = 0; k < c.ptot; ++k) s->fsol[c.plist[k].matid - 1] = c.plist[k].pressure;
    // the solver the parameters name: BiCGStab, or fgmres as the reference's
    // live ppesolve (solver.f90:306-350)
    const auto spmv = [&](const std::vector<double>& b, std::vector<double>& r) { spmv2(s, b, r); };
    int st = (s->P.ppe_solver == BS_SOLVER_FGMRES)
                 ? fgmres(n, spmv, s->fvec, s->fsol, tol, maxit, std::max(1, (int)s->P.ppe_restart), rule, iters,
                          relres)
                 : bicgstab(n, spmv, s->fvec, s->fsol, tol, maxit, rule, iters, relres);
    // pressure scatter, isph.f90:468-486
    for_interior(s, [&](int i, int j) {
        Cell& c = s->C(i, j);
        for (int k = 0; k < c.ptot; ++k) c.plist[k].pressure = s->fsol[c.plist[k].matid - 1];
    });
    s->last_iters = *iters;
    s->last_relres = *relres;
    if (st) s->err |= BS_ERR_NOT_CONVERGED;
    return st;
}

// --------------------------------------------------------------- comp_vel
// integrator.f90:705-843
void comp_vel(or_scene* s) {
    const double dt = s->dt;
    for_interior(s, [&](int i, int j) {
        Cell& c = s->C(i, j);
        for (int k = 0; k < c.ptot; ++k) {
            Particle& p = c.plist[k];
            Props& pp = c.pplist[k];
            const Verlet& L = c.list[k];
            if ((p.tid == 3) && !p.buffer) {
                p.vx = 0.0;
                p.vy = 0.0;
                for (int m = 0; m < L.count; ++m) {
                    const Cell& oc = s->cells[L.nh[m].cell];
                    const Particle& x = oc.plist[L.nh[m].slot];
                    const Props& y = oc.pplist[L.nh[m].slot];
                    const double z1 = L.kx[m], z2 = L.ky[m];
                    double t1;
                    if (x.tid == 3)
                        t1 = 2 * ((x.mass / x.density) * (pp.porosity * pp.porosity) *
                                  ((x.pressure * p.density / pp.porosity) + (p.pressure * x.density / y.porosity)) *
                                  (pp.coff[0] * z1 + pp.coff[1] * z2)) /
                             ((p.density) * ((p.density / pp.porosity) + (x.density / y.porosity)));
                    else
                        t1 = ((x.mass / x.density) * (pp.porosity * pp.porosity) * (x.pressure + p.pressure) *
                              (pp.coff[0] * z1 + pp.coff[1] * z2)) / p.density;
                    p.vx = p.vx - t1 * dt;
                    if (x.tid == 3)
                        t1 = 2 * ((x.mass / x.density) * (pp.porosity * pp.porosity) *
                                  ((x.pressure * p.density / pp.porosity) + (p.pressure * x.density / y.porosity)) *
                                  (pp.coff[2] * z1 + pp.coff[3] * z2)) /
                             ((p.density) * ((p.density / pp.porosity) + (x.density / y.porosity)));
                    else
                        t1 = ((x.mass / x.density) * (pp.porosity * pp.porosity) * (x.pressure + p.pressure) *
                              (pp.coff[2] * z1 + pp.coff[3] * z2)) / p.density;
                    p.vy = p.vy - t1 * dt;
                }
                p.vx = p.vxs + p.vx;
                p.vy = p.vys + p.vy;
                pp.vel = std::sqrt(p.vx * p.vx + p.vy * p.vy) / pp.porosity;
            }
            if (p.buffer) {
                p.vx = p.vxs;
                p.vy = 0.0;
            }
        }
    });
    for_interior(s, [&](int i, int j) {   // per-cell maxima (831-841): stale when the cell is empty
        Cell& c = s->C(i, j);
        if (c.ptot != 0) {
            double mv = 0, me = 0;
            for (int k = 0; k < c.ptot; ++k) {
                mv = std::max(mv, std::fabs(c.pplist[k].vel));
                me = std::max(me, std::fabs(c.pplist[k].nut));
            }
            c.maxvel = mv;
            c.maxeddy = me;
        }
    });
}

// --------------------------------------------------------------- comp_pos
// integrator.f90:845-883; the release window (8 prrealx + brrealx + 0.001,
// xrcutoff) of 865-872 is the parameter pair buf_release_lo / hi
void comp_pos(or_scene* s) {
    const double dt = s->dt;
    for_interior(s, [&](int i, int j) {
        Cell& c = s->C(i, j);
        for (int k = 0; k < c.ptot; ++k) {
            Particle& p = c.plist[k];
            const Props& pp = c.pplist[k];
            if (p.tid == 3) {
                p.x = (p.x + p.xs + dt * p.vx / pp.porosity) / 2.0;
                p.y = (p.y + p.ys + dt * p.vy / pp.porosity) / 2.0;
                if (p.buffer && (p.x > s->P.buf_release_lo) && (p.x < s->P.buf_release_hi)) p.buffer = false;
            }
        }
    });
}

// --------------------------------------------------------------- freesurf
// isph.f90:49-86 (many threads write .true. to shared neighbours: benign)
void freesurf(or_scene* s) {
    const double thr = s->P.lamfs * s->P.maxdivr;
    for_interior(s, [&](int i, int j) {
        Cell& c = s->C(i, j);
        for (int k = 0; k < c.ptot; ++k) {
            const Particle& p = c.plist[k];
            if ((p.tid == 3) && !p.buffer && c.pplist[k].gradvx <= thr) {
                const Verlet& L = c.list[k];
                for (int m = 0; m < L.count; ++m) {
                    Particle& x = s->cells[L.nh[m].cell].plist[L.nh[m].slot];
#pragma omp atomic write
                    x.vicinity = true;
                }
            }
        }
    });
}

// ------------------------------------------------------------- opt2_shift
// part_shift.f90:12-191
void opt2_shift(or_scene* s) {
    const double csh = s->P.csh, maxshift = s->P.maxshift, dl = s->dl, h1 = s->h;
    unsigned errs = 0;
    for_interior(s, [&](int i, int j) {
        Cell& c = s->C(i, j);
        for (int k = 0; k < c.ptot; ++k) {
            Particle& p = c.plist[k];
            const Props& pp = c.pplist[k];
            const Verlet& L = c.list[k];
            if (!((p.tid == 3) && !p.buffer)) continue;
            double xs = 0.0, ys = 0.0;
            const double heff = h1;
            if (L.count != 0) {
                double normx = 0.0, normy = 0.0;
                for (int m = 0; m < L.count; ++m) {
                    const Particle& x = s->cells[L.nh[m].cell].plist[L.nh[m].slot];
                    normx = normx - (pp.coff[0] * L.kx[m] + pp.coff[1] * L.ky[m]) * (x.mass / x.density);
                    normy = normy - (pp.coff[2] * L.kx[m] + pp.coff[3] * L.ky[m]) * (x.mass / x.density);
                }
                double t1 = std::sqrt(normx * normx + normy * normy);
                normx = normx / t1;
                normy = normy / t1;
                normx = 0.0;   // merge(0.0_dp,0.0_dp,...) (67-68)
                normy = 0.0;
                const int pint = 0;   // (69)
                const double frac = p.free ? 0.01 : 1.0;   // (70)
                for (int m = 0; m < L.count; ++m) {
                    const Particle& x = s->cells[L.nh[m].cell].plist[L.nh[m].slot];
                    const double w4 = 0.0;   // (Wab(r)/Wab(dl))**4 is multiplied by 0.2*pint = 0
                    xs = xs - csh * (heff * heff) * frac * ((1 - normx * normx) * L.kx[m] - normx * normy * L.ky[m]) *
                                  (x.mass / x.density) * (1.0 + 0.20 * pint * w4);
                }
                p.xs = std::min(std::fabs(xs), maxshift * dl) * xs / std::fabs(xs);
                for (int m = 0; m < L.count; ++m) {
                    const Particle& x = s->cells[L.nh[m].cell].plist[L.nh[m].slot];
                    const double w4 = 0.0;
                    ys = ys - csh * (heff * heff) * frac * (-normx * normy * L.kx[m] + (1 - normy * normy) * L.ky[m]) *
                                  (x.mass / x.density) * (1.0 + 0.20 * pint * w4);
                }
                p.ys = std::min(std::fabs(ys), maxshift * dl) * ys / std::fabs(ys);
                if (xs == 0.0 || ys == 0.0) {
#pragma omp atomic
                    errs |= BS_ERR_ZERO_SHIFT;
                }
                double a1 = 0.0, a2 = 0.0;
                for (int m = 0; m < L.count; ++m) {
                    const Particle& x = s->cells[L.nh[m].cell].plist[L.nh[m].slot];
                    a1 = a1 + ((pp.coff[0] * L.kx[m] + pp.coff[1] * L.ky[m]) * (x.vx - p.vx)) * (x.mass / x.density);
                    a2 = a2 + ((pp.coff[2] * L.kx[m] + pp.coff[3] * L.ky[m]) * (x.vx - p.vx)) * (x.mass / x.density);
                }
                p.vxs = a1 * xs + a2 * ys;
                a1 = 0.0;
                a2 = 0.0;
                for (int m = 0; m < L.count; ++m) {
                    const Particle& x = s->cells[L.nh[m].cell].plist[L.nh[m].slot];
                    a1 = a1 + ((pp.coff[0] * L.kx[m] + pp.coff[1] * L.ky[m]) * (x.vy - p.vy)) * (x.mass / x.density);
                    a2 = a2 + ((pp.coff[2] * L.kx[m] + pp.coff[3] * L.ky[m]) * (x.vy - p.vy)) * (x.mass / x.density);
                }
                p.vys = a1 * xs + a2 * ys;
            } else {
#pragma omp atomic
                errs |= BS_ERR_NO_NEIGHBOUR;
            }
        }
    });
    s->err |= errs;
    for_interior(s, [&](int i, int j) {   // apply (172-189)
        Cell& c = s->C(i, j);
        for (int k = 0; k < c.ptot; ++k) {
            Particle& p = c.plist[k];
            if ((p.tid == 3) && !p.buffer) {
                p.x = p.x + p.xs;
                p.y = p.y + p.ys;
                p.vx = p.vx + p.vxs;
                p.vy = p.vy + p.vys;
            }
        }
    });
}

// ---------------------------------------------------------- densityupdate
// scalar.f90:399-426
void densityupdate(or_scene* s) {
    const double rhomax = s->P.rhomax, rhomin = s->P.rhomin;
    for_interior(s, [&](int i, int j) {
        Cell& c = s->C(i, j);
        for (int k = 0; k < c.ptot; ++k) {
            Particle& p = c.plist[k];
            if (p.tid == 3) {
                p.oden = 0.5 * (rhomax + rhomin) + p.con * (rhomax - rhomin);
                p.mass = p.oden * p.ovol;
                p.density = p.oden * c.pplist[k].porosity;
            }
        }
    });
}

// --------------------------------------------------------------- timestep
// integrator.f90:885-953
void timestep(or_scene* s) {
    double umax = 0.0, numax = 0.0;
    for (int j = 2; j <= s->cellx - 1; ++j)
        for (int i = 2; i <= s->celly - 1; ++i) {
            umax = std::max(umax, s->C(i, j).maxvel);
            numax = std::max(numax, s->C(i, j).maxeddy);
        }
    s->umax = umax;
    const double sig1 = s->P.sig1, dl = s->dl, mu = s->P.mu, rho = s->P.rho, t = s->t;
    if (s->P.adaptive_dt) {
        if (t <= 1.0)
            s->dt = std::min({sig1 * (dl) / umax, sig1 * ((dl) * (dl)) / ((mu / rho) + numax), 0.0010});
        else if ((t > 1.0) && (t <= 2.50))
            s->dt = (double)std::min({(float)(sig1 * (dl) / umax), (float)(sig1 * ((dl) * (dl)) * rho / mu), 0.002f});
        else if ((t > 3.0) && (t <= 4.0))
            s->dt = (double)std::min({(float)(sig1 * (dl) / umax), (float)(sig1 * ((dl) * (dl)) * rho / mu), 0.004f});
        else
            s->dt = std::min({sig1 * (dl) / umax, sig1 * ((dl) * (dl)) / ((mu / rho) + numax), 0.0050});
    }
    if (!std::isfinite(numax) || std::isnan(numax)) numax = 0.0;
    s->numax = numax;
    double dtsol = sig1 * (dl * dl) / (SP_1EM9 + numax / s->P.tschmidt);
    int solsteps = 1;
    if (dtsol < s->dt) {
        solsteps = (int)std::ceil(s->dt / dtsol);
        dtsol = s->dt / solsteps;
    }
    dtsol = (dtsol < s->dt) ? dtsol : s->dt;
    s->dtsol = dtsol;
    s->solsteps = solsteps;
}

// ------------------------------------------------------ scalar transport
// scalart_anisotropic scalar.f90:242-362 and scalarupdate 364-397
void scalar_substep(or_scene* s) {
    const double al = 0.0025, at = 0.00025, Dm = SP_1EM9, threshpor = 0.7;
    const double lam = s->lam, h1 = s->h, dl = s->dl, dt = s->dt, tsch = s->P.tschmidt;
    for_interior(s, [&](int i, int j) {
        Cell& c = s->C(i, j);
        for (int k = 0; k < c.ptot; ++k) {
            const Particle& p = c.plist[k];
            Props& pp = c.pplist[k];
            const Verlet& L = c.list[k];
            if (p.tid != 3) continue;
            pp.cdiff = 0.0;
            const double con1 = p.con;
            for (int m = 0; m < L.count; ++m) {
                const Particle& x = s->cells[L.nh[m].cell].plist[L.nh[m].slot];
                const Props& y = s->cells[L.nh[m].cell].pplist[L.nh[m].slot];
                const double vi = std::sqrt(p.vx * p.vx + p.vy * p.vy) / pp.porosity;
                if (x.tid != 3) continue;
                const double con2 = x.con;
                const double vj = std::sqrt(x.vx * x.vx + x.vy * x.vy) / y.porosity;
                const bool pz = (pp.porosity < threshpor) && (y.porosity < threshpor);
                const double Dxxi = pz ? (p.vx) / (std::sqrt((al * vi) + Dm) * vi * pp.porosity) : Dm + pp.nut / tsch;
                const double Dxyi = pz ? (p.vy) / (std::sqrt((al * vi) + Dm) * vi * pp.porosity) : 0.0;
                const double Dyxi = pz ? (-p.vy) / (std::sqrt((at * vi) + Dm) * vi * pp.porosity) : 0.0;
                const double Dyyi = pz ? (p.vx) / (std::sqrt((at * vi) + Dm) * vi * pp.porosity) : Dm + pp.nut / tsch;
                const double Dxxj = pz ? (x.vx) / (std::sqrt((al * vj) + Dm) * vj * y.porosity) : Dm + y.nut / tsch;
                const double Dxyj = pz ? (x.vy) / (std::sqrt((al * vj) + Dm) * vj * y.porosity) : 0.0;
                const double Dyxj = pz ? (-x.vy) / (std::sqrt((at * vj) + Dm) * vj * y.porosity) : 0.0;
                const double Dyyj = pz ? (x.vx) / (std::sqrt((at * vj) + Dm) * vj * y.porosity) : Dm + y.nut / tsch;
                double t1x, t1y;
                const double dm = L.dist[m];
                if (pz) {
                    const double p_dist = 1.0 / dm;
                    t1x = sq(((Dxxi + Dxxj) * (p.x - x.x) * p_dist * 0.5) + ((Dxyi + Dxyj) * (p.y - x.y) * p_dist * 0.5)) +
                          sq(((Dyxi + Dyxj) * (p.x - x.x) * p_dist * 0.5) + ((Dyyi + Dyyj) * (p.y - x.y) * p_dist * 0.5));
                    t1x = 1.0 / t1x;
                    const double cap = 0.12 * (dl * dl) / dt;
                    t1x = (t1x <= cap) ? t1x : cap;
                    t1y = t1x;
                } else {
                    if ((pp.nut < SP_1EM6) && (y.nut < SP_1EM6)) t1x = (Dxxi + Dxxj) * 0.50;
                    else t1x = 2 * Dxxi * Dxxj / (Dxxi + Dxxj);
                    t1y = t1x;
                }
                const double t2 = 1.0;
                const double t3 = (p.ovol) * (pp.porosity + y.porosity) / (pp.porosity * y.porosity);
                const double gx = Wabx(x, p, dm, h1), gy = Waby(x, p, dm, h1);
                pp.cdiff = pp.cdiff + (t1x * t2 * t3 * (con1 - con2) * (p.x - x.x) * gx / (dm * dm + lam)) +
                           (t1y * t2 * t3 * (con1 - con2) * (p.y - x.y) * gy / (dm * dm + lam));
            }
        }
    });
    const double dts = s->dtsol;
    for_interior(s, [&](int i, int j) {
        Cell& c = s->C(i, j);
        for (int k = 0; k < c.ptot; ++k) {
            Particle& p = c.plist[k];
            if (p.tid == 3) {
                p.con = p.con + c.pplist[k].cdiff * dts;
                if (p.buffer && (p.x < 1.6)) p.con = 0.5;
            }
        }
    });
}

// Initial state: what the reference's warm-up leaves for the production loop
// (ids, neighbour lists, porosity, eddy viscosity, per-cell maxima, timestep).
// --------------------------------------------------------------- WCSPH
// wcsph.f90 (compiled into no reference executable).  co, t_gam, delt and
// the still-water level come from the parameters (co is never set by the
// reference, setup.f90:134).

// hydrostatic Tait density at height y (the term2 expression, wcsph.f90:78-82)
double hyd_density(const or_scene* s, double y) {
    const double rho = s->P.rho, co = s->P.wc_c0, gam = s->P.wc_gamma;
    return rho * std::pow(((((s->P.wc_ysurf - y) * rho) * std::fabs(s->P.g)) * gam) / (rho * (co * co)) + 1.0,
                          1.0 / gam);
}

// calmasscons, wcsph.f90:65-129.  term2 is both the hydrostatic density
// difference of the current pair and the y accumulator: the reference
// overwrites it with the pair's hydrostatic difference at every neighbour,
// so only the last neighbour's y contribution survives; kept as written.
void calmasscons(or_scene* s) {
    const double rho = s->P.rho, co = s->P.wc_c0, delt = s->P.wc_delta, h1 = s->h, lam = s->lam;
    const double dt = s->dt;
    for_interior(s, [&](int i, int j) {
        Cell& c = s->C(i, j);
        for (int k = 0; k < c.ptot; ++k) {
            Particle& p = c.plist[k];
            if (!(p.tid > 2)) continue;
            const Props& pp = c.pplist[k];
            const Verlet& L = c.list[k];
            double term1 = 0.0, term2 = 0.0;
            for (int m = 0; m < L.count; ++m) {
                const Particle& x = s->cells[L.nh[m].cell].plist[L.nh[m].slot];
                const double r = L.dist[m];
                const double wx = Wabx(x, p, r, h1), wy = Waby(x, p, r, h1);
                const double gx = pp.coff[0] * wx + pp.coff[1] * wy;
                const double gy = pp.coff[2] * wx + pp.coff[3] * wy;
                const double hd = hyd_density(s, x.y) - hyd_density(s, p.y);
                // as written: term2 doubles as hd, delta term along (r_i - r_j)
                // (anti-diffusive); corrected: own y sum, along (r_j - r_i)
                const double sg = (s->P.wc_form == 0) ? 1.0 : -1.0;
                if (s->P.wc_form == 0) term2 = hd;
                term1 = term1 - ((x.mass * (x.vx - p.vx)) * gx) * (p.density / x.density) +
                        ((((((delt * 2) * h1) * co) * (x.density - p.density - hd)) * (sg * (p.x - x.x))) * gx) *
                            (x.mass / x.density) / (r * r + lam);
                term2 = term2 - ((x.mass * (x.vy - p.vy)) * gy) * (p.density / x.density) +
                        ((((((delt * 2) * h1) * co) * (x.density - p.density - hd)) * (sg * (p.y - x.y))) * gy) *
                            (x.mass / x.density) / (r * r + lam);
            }
            p.tden = p.density + (term1 + term2) * dt;
        }
    });
}

// updateden, wcsph.f90:131-154
void updateden(or_scene* s) {
    for_interior(s, [&](int i, int j) {
        Cell& c = s->C(i, j);
        for (int k = 0; k < c.ptot; ++k)
            if (c.plist[k].tid > 2) c.plist[k].density = c.plist[k].tden;
    });
}

// dentopress, wcsph.f90:35-63 (Tait equation of state, no tension)
void dentopress(or_scene* s) {
    const double rho = s->P.rho, co = s->P.wc_c0, gam = s->P.wc_gamma;
    for_interior(s, [&](int i, int j) {
        Cell& c = s->C(i, j);
        for (int k = 0; k < c.ptot; ++k) {
            Particle& p = c.plist[k];
            if (!(p.tid > 2)) continue;
            p.pressure = (rho * (co * co)) * (std::pow(p.density / rho, gam) - 1) / gam;
            if (p.pressure < 0.0) {
                p.pressure = 0.0;
                p.density = rho;
            }
        }
    });
}

// presstoden, wcsph.f90:13-33
void presstoden(or_scene* s) {
    const double rho = s->P.rho, co = s->P.wc_c0, gam = s->P.wc_gamma;
    for_interior(s, [&](int i, int j) {
        Cell& c = s->C(i, j);
        for (int k = 0; k < c.ptot; ++k) {
            Particle& p = c.plist[k];
            p.density = rho * std::pow((p.pressure * gam / (rho * (co * co))) + 1, 1 / gam);
        }
    });
}

// Wall and ghost pressure of the WCSPH step (this library's boundary rule;
// the reference has none): Shepard average over fluid neighbours of
// p_f + rho_f |g| (y_f - y_w), 0 without fluid neighbours.
void wall_pressure(or_scene* s) {
    const double ag = std::fabs(s->P.g), h1 = s->h;
    for_interior(s, [&](int i, int j) {
        Cell& c = s->C(i, j);
        for (int k = 0; k < c.ptot; ++k) {
            Particle& p = c.plist[k];
            if (p.tid == 3) continue;
            const Verlet& L = c.list[k];
            double num = 0.0, den = 0.0;
            for (int m = 0; m < L.count; ++m) {
                const Particle& x = s->cells[L.nh[m].cell].plist[L.nh[m].slot];
                if (x.tid != 3) continue;
                const double w = Wab(L.dist[m], h1);
                num += (x.pressure + x.density * ag * (x.y - p.y)) * w;
                den += w;
            }
            p.pressure = den > 0.0 ? num / den : 0.0;
        }
    });
}

// boun_vel, integrator.f90:394-457 (compiled, never called): wall and ghost
// particles take minus the Shepard average of their fluid neighbours'
// velocity, divided only when the Shepard sum reaches 1e-6 (single literal);
// vxs = vys = 0.
void boun_vel(or_scene* s) {
    const double h1 = s->h;
    for_interior(s, [&](int i, int j) {
        Cell& c = s->C(i, j);
        for (int k = 0; k < c.ptot; ++k) {
            Particle& p = c.plist[k];
            if (p.tid > 2) continue;
            double t1 = 0.0;
            p.vx = 0.0;
            p.vy = 0.0;
            p.vxs = 0.0;
            p.vys = 0.0;
            const Verlet& L = c.list[k];
            for (int m = 0; m < L.count; ++m) {
                const Particle& x = s->cells[L.nh[m].cell].plist[L.nh[m].slot];
                if (x.tid != 3) continue;
                const double w = Wab(L.dist[m], h1);
                p.vx = p.vx - x.mass * w * x.vx / x.density;
                p.vy = p.vy - x.mass * w * x.vy / x.density;
                t1 = t1 + x.mass * w / x.density;
            }
            if (t1 >= SP_1EM6) {
                p.vx = p.vx / t1;
                p.vy = p.vy / t1;
            }
        }
    });
}

// coll_pos_shift (mode 0, part_shift.f90:193-292) and coll_shift (mode 1,
// 294-410), compiled but never called.  Pass 1: every particle's xs, ys
// (mode 0) or vxs, vys (mode 1) set to 0; for fluid particles with
// neighbours, gradvx >= 0.7 and not in a buffer, per axis a mass-weighted
// push from the neighbours closer than the collision distance
// dcol = pr/sqrt(phi_i) + (fluid ? pr : br)/sqrt(phi_j) -- the overlap
// (mode 0) or the approaching relative pore velocity (mode 1, t3 < 0) --
// over m_i + sum m_j.  Pass 2: mode 0 moves those particles by (xs, ys);
// mode 1 adds phi (vxs, vys) to the velocity of every fluid particle not in
// a buffer.  cr = 0, disfac = 1 as the module's parameters; merge() adds
// 0.0 where the condition fails, so the sums are kept the same way.
void collision_shift(or_scene* s, int mode, double prx, double pry, double brx, double bry) {
    const double cr = 0.0, disfac = 1.0;
    for_interior(s, [&](int i, int j) {
        Cell& c = s->C(i, j);
        for (int k = 0; k < c.ptot; ++k) {
            Particle& p = c.plist[k];
            const Props& pp = c.pplist[k];
            const Verlet& L = c.list[k];
            double& sx = mode ? p.vxs : p.xs;
            double& sy = mode ? p.vys : p.ys;
            sx = 0.0;
            sy = 0.0;
            if (!((L.count != 0) && (pp.gradvx >= 0.70) && (p.tid == 3) && !p.buffer)) continue;
            for (int ax = 0; ax < 2; ++ax) {
                const double pr = ax ? pry : prx, br = ax ? bry : brx;
                double t1 = 0.0, t2 = 0.0;
                for (int m = 0; m < L.count; ++m) {
                    const Cell& oc = s->cells[L.nh[m].cell];
                    const Particle& x = oc.plist[L.nh[m].slot];
                    const Props& y = oc.pplist[L.nh[m].slot];
                    const double d = L.dist[m];
                    const double dcol = disfac * (pr * (1.0 / std::sqrt(pp.porosity)) +
                                                  (x.tid == 3 ? pr : br) * (1.0 / std::sqrt(y.porosity)));
                    t1 = t1 + x.mass;
                    const double rel = ax ? (p.y - x.y) : (p.x - x.x);
                    double term = 0.0;
                    if (mode == 0) {
                        if (d < dcol) term = (-1.0 * (x.mass * (1.0 + cr) * (d - dcol))) * (rel / d);
                    } else {
                        const double t3 = (p.x - x.x) * (p.vx * (1.0 / pp.porosity) - x.vx * (1.0 / y.porosity)) +
                                          (p.y - x.y) * (p.vy * (1.0 / pp.porosity) - x.vy * (1.0 / y.porosity));
                        if ((d < dcol) && (t3 < 0.0)) term = (-1.0 * (x.mass * (1.0 + cr) * t3)) * (rel / (d * d));
                    }
                    t2 = t2 + term;
                }
                (ax ? sy : sx) = t2 / (p.mass + t1);
            }
        }
    });
    for_interior(s, [&](int i, int j) {
        Cell& c = s->C(i, j);
        for (int k = 0; k < c.ptot; ++k) {
            Particle& p = c.plist[k];
            const Props& pp = c.pplist[k];
            if (p.tid != 3 || p.buffer) continue;
            if (mode == 0) {
                if (pp.gradvx >= 0.70) {
                    p.x = p.x + p.xs;
                    p.y = p.y + p.ys;
                }
            } else {
                p.vx = p.vx + p.vxs * pp.porosity;
                p.vy = p.vy + p.vys * pp.porosity;
            }
        }
    });
}

// invertmat3D, functions.f90:134-165: adjugate over the determinant; err when
// det < 1e-5 (single literal) or not finite
bool invertmat3D(double a[3][3]) {
    const double det = a[0][0] * (a[1][1] * a[2][2] - a[2][1] * a[1][2]) -
                       a[0][1] * (a[1][0] * a[2][2] - a[2][0] * a[1][2]) +
                       a[0][2] * (a[1][0] * a[2][1] - a[2][0] * a[1][1]);
    if (det < (double)1e-5f || !std::isfinite(det)) {
        for (int u = 0; u < 3; ++u)
            for (int v = 0; v < 3; ++v) a[u][v] = 0.0;
        return true;
    }
    double r[3][3];
    r[0][0] = (a[1][1] * a[2][2] - a[2][1] * a[1][2]);
    r[1][0] = -(a[0][1] * a[2][2] - a[2][1] * a[0][2]);
    r[2][0] = (a[0][1] * a[1][2] - a[1][1] * a[0][2]);
    r[0][1] = -(a[1][0] * a[2][2] - a[2][0] * a[1][2]);
    r[1][1] = (a[0][0] * a[2][2] - a[2][0] * a[0][2]);
    r[2][1] = -(a[0][0] * a[1][2] - a[1][0] * a[0][2]);
    r[0][2] = (a[1][0] * a[2][1] - a[2][0] * a[1][1]);
    r[1][2] = -(a[0][0] * a[2][1] - a[2][0] * a[0][1]);
    r[2][2] = (a[1][1] * a[0][0] - a[1][0] * a[0][1]);
    for (int u = 0; u < 3; ++u)
        for (int v = 0; v < 3; ++v) a[u][v] = r[u][v] / det;
    return false;
}

// comp_ghost + ghost_en, mls.f90:114-263 (not compiled).  Wall and ghost
// particles with neighbours take minus the Shepard average of their fluid
// neighbours' velocity, tke and nut (list2 of the module is never built: the
// neighbour list restricted to fluid stands in; a zero Shepard sum leaves 0
// where the module would divide by it).  use_mls: the module's commented-out
// moving-least-squares branch for the velocity -- weights
// W (b1 + b2 dx + b3 dy) V with b the first column of the inverse moment
// matrix over all neighbours (Wmls, mls.f90:16-111) -- where invertmat3D
// succeeds, the Shepard average elsewhere.
void ghost(or_scene* s, bool use_mls) {
    const double h1 = s->h;
    for_interior(s, [&](int i, int j) {
        Cell& c = s->C(i, j);
        for (int k = 0; k < c.ptot; ++k) {
            Particle& p = c.plist[k];
            Props& pp = c.pplist[k];
            if (p.tid > 2) continue;
            p.vx = 0.0;
            p.vy = 0.0;
            pp.tke = 0.0;
            pp.nut = 0.0;
            const Verlet& L = c.list[k];
            if (L.count == 0) continue;
            bool err = true;
            double b[3] = {0, 0, 0};
            if (use_mls) {
                double a[3][3] = {{0, 0, 0}, {0, 0, 0}, {0, 0, 0}};
                for (int m = 0; m < L.count; ++m) {
                    const Particle& x = s->cells[L.nh[m].cell].plist[L.nh[m].slot];
                    const double w = Wab(L.dist[m], h1), v = x.mass / x.density;
                    const double dx = p.x - x.x, dy = p.y - x.y;
                    a[0][0] = a[0][0] + w * v;
                    a[1][0] = a[1][0] + w * dx * v;
                    a[2][0] = a[2][0] + w * dy * v;
                    a[0][1] = a[0][1] + w * dx * v;
                    a[1][1] = a[1][1] + w * (dx * dx) * v;
                    a[2][1] = a[2][1] + w * dx * dy * v;
                    a[0][2] = a[0][2] + w * dy * v;
                    a[1][2] = a[1][2] + w * dx * dy * v;
                    a[2][2] = a[2][2] + w * (dy * dy) * v;
                }
                err = invertmat3D(a);
                if (!err) {
                    b[0] = a[0][0];
                    b[1] = a[1][0];
                    b[2] = a[2][0];
                }
            }
            double t1 = 0.0, te = 0.0;
            for (int m = 0; m < L.count; ++m) {
                const Particle& x = s->cells[L.nh[m].cell].plist[L.nh[m].slot];
                if (x.tid != 3) continue;
                const Props& y = s->cells[L.nh[m].cell].pplist[L.nh[m].slot];
                const double w = Wab(L.dist[m], h1);
                if (!err) {
                    const double q = w * (b[0] + b[1] * (p.x - x.x) + b[2] * (p.y - x.y)) * (x.mass / x.density);
                    p.vx = p.vx - x.vx * q;
                    p.vy = p.vy - x.vy * q;
                } else {
                    p.vx = p.vx - w * x.vx * x.mass / x.density;
                    p.vy = p.vy - w * x.vy * x.mass / x.density;
                    t1 = t1 + x.mass * w / x.density;
                }
                pp.tke = pp.tke - w * y.tke * x.mass / x.density;
                pp.nut = pp.nut - w * y.nut * x.mass / x.density;
                te = te + x.mass * w / x.density;
            }
            if (err && t1 > 0.0) {
                p.vx = p.vx / t1;
                p.vy = p.vy / t1;
            }
            if (te > 0.0) {
                pp.tke = pp.tke / te;
                pp.nut = pp.nut / te;
            }
        }
    });
}

void prime(or_scene* s, bool rule = true) {
    resetid(s);
    neighbour(s);
    effpor(s);
    eddyvis(s);
    for_interior(s, [&](int i, int j) {
        Cell& c = s->C(i, j);
        double mv = 0, me = 0;
        for (int k = 0; k < c.ptot; ++k) {
            const Particle& p = c.plist[k];
            Props& pp = c.pplist[k];
            if (p.tid == 3 && !p.buffer) pp.vel = std::sqrt(p.vx * p.vx + p.vy * p.vy) / pp.porosity;
            mv = std::max(mv, std::fabs(pp.vel));
            me = std::max(me, std::fabs(pp.nut));
        }
        c.maxvel = mv;
        c.maxeddy = me;
    });
    if (rule) timestep(s);
}

// one production step, main.f90:199-272 (buffers excluded)
// remove_bufferN (internal.f90:516-584) then insert_bufferN (447-514) of one
// zone: entry cells drop their buffer particles at or beyond remove_x (plist
// compacted, pplist left in place -- the slot keeps its properties), then
// every template particle inside an entry cell is appended to it in template
// order.  A slot beyond the cell's count before the exchange starts from the
// properties' defaults (the reference would read whatever the slot last held).
void buffer_exchange(or_scene* s, int z) {
    OrZone& Z = s->zones[z];
    std::vector<int> oldn(Z.cells.size());
    for (size_t q = 0; q < Z.cells.size(); ++q) {
        Cell& c = s->C(Z.cells[q].first, Z.cells[q].second);
        oldn[q] = c.ptot;
        int keep = 0;
        for (int k = 0; k < c.ptot; ++k) {
            const Particle& p = c.plist[k];
            const bool rm = p.buffer && (Z.side > 0 ? (p.x >= Z.remove_x) : (p.x <= Z.remove_x));
            if (!rm) c.plist[keep++] = p;
        }
        c.ptot = keep;
    }
    for (size_t q = 0; q < Z.cells.size(); ++q) {
        Cell& c = s->C(Z.cells[q].first, Z.cells[q].second);
        for (const Particle& t : Z.tmpl) {
            if (!((t.x >= c.xleft) && (t.x < c.xright) && (t.y >= c.ybot) && (t.y < c.ytop))) continue;
            const int k = c.ptot++;
            if ((int)c.plist.size() < c.ptot) c.plist.resize(c.ptot);
            if ((int)c.pplist.size() < c.ptot) c.pplist.resize(c.ptot);
            c.plist[k] = t;
            if (k >= oldn[q]) c.pplist[k] = Props();
        }
    }
}

// main.f90:218-234: zone z exchanges when (told + phase) < k*period <= (t + phase)
void buffer_schedule(or_scene* s, double told) {
    for (int z = 0; z < 2; ++z) {
        OrZone& Z = s->zones[z];
        if (!Z.set || !(Z.period > 0)) continue;
        const double kp = (double)Z.next_k * Z.period;
        if (((told + Z.phase) < kp) && ((s->t + Z.phase) >= kp)) {
            buffer_exchange(s, z);
            Z.next_k += 1;
        }
    }
}

// one step of main.f90's loops; flags (BS_STEP_*) select the parts the
// settling phases (main.f90:39-67, 95-155) leave out
void step(or_scene* s, int flags = BS_STEP_ALL) {
    const double told = s->t;
    s->t = s->t + s->dt;
    if (s->P.scalar_on && (flags & BS_STEP_SCALAR))
        for (int j1 = 1; j1 <= s->solsteps; ++j1) scalar_substep(s);
    if (flags & BS_STEP_BUFFERS) buffer_schedule(s, told);
    projection(s);
    cellshift(s, false);
    resetid(s);
    neighbour(s);
    effpor(s);
    eddyvis(s);
    int_vel(s);
    ppe_assemble(s);
    int it;
    double rr;
    ppe_solve(s, s->P.ppe_tol, s->P.ppe_maxit, s->P.ppe_stop, &it, &rr);
    comp_vel(s);
    comp_pos(s);
    cellshift(s, true);
    neighbour(s);
    freesurf(s);
    effpor(s);
    opt2_shift(s);
    if (flags & BS_STEP_DENSITY) densityupdate(s);
    timestep(s);
    if (flags & BS_STEP_EDDY_END) eddyvis(s);
}

// WCSPH step: the production step with continuity + Tait EOS + wall
// pressure in place of the PPE, density kept from the continuity equation
void wcsph_step(or_scene* s) {
    const double told = s->t;
    s->t = s->t + s->dt;
    if (s->P.scalar_on)
        for (int j1 = 1; j1 <= s->solsteps; ++j1) scalar_substep(s);
    buffer_schedule(s, told);
    projection(s);
    cellshift(s, false);
    resetid(s);
    neighbour(s);
    effpor(s, true);
    eddyvis(s);
    int_vel(s);
    calmasscons(s);
    updateden(s);
    dentopress(s);
    wall_pressure(s);
    comp_vel(s);
    comp_pos(s);
    cellshift(s, true);
    neighbour(s);
    freesurf(s);
    effpor(s, true);
    opt2_shift(s);
    timestep(s);
    eddyvis(s);
}

template <class T>
void put(T* dst, size_t q, T v) { if (dst) dst[q] = v; }

}  // namespace

// ============================================================== C API
extern "C" {

or_scene* or_create(const bs_params* p, const bs_state* st, const bs_grains* gr) {
    or_scene* s = new or_scene();
    s->P = *p;
    s->cellx = p->cellx;
    s->celly = p->celly;
    s->h = p->h;
    s->dl = p->dl;
    s->lam = 0.0010 * (p->h * p->h);   // setup.f90:82
    s->cw = 4.0 * p->h;
    s->dt = p->dt;
    s->t = p->t0;
    s->cells.resize((size_t)s->cellx * s->celly);
    for (int j = 1; j <= s->cellx; ++j)
        for (int i = 1; i <= s->celly; ++i) {
            Cell& c = s->C(i, j);
            c.xleft = xleft_of(s, j);
            c.xright = xright_of(s, j);
            c.ybot = ybot_of(s, i);
            c.ytop = ytop_of(s, i);
        }
    // distribute: walls first (btot) in input order, then fluid in input order
    // (boundary.f90:140-190 then internal.f90:73-95)
    for (int pass = 0; pass < 2; ++pass)
        for (int q = 0; q < st->n; ++q) {
            const bool wall = st->tid[q] != 3;
            if ((pass == 0) != wall) continue;
            int ci, cj;
            if (!locate(s, st->x[q], st->y[q], &ci, &cj)) { s->err |= BS_ERR_LOST_PARTICLE; continue; }
            Particle P;
            P.x = st->x[q]; P.y = st->y[q]; P.vx = st->vx[q]; P.vy = st->vy[q];
            P.pressure = st->p[q]; P.mass = st->mass[q]; P.density = st->rho[q]; P.oden = st->oden[q];
            P.ovol = st->ovol[q]; P.con = st->con[q]; P.tid = st->tid[q]; P.pid = st->pid[q];
            P.free = st->flags[q] & BS_FLAG_FREE; P.vicinity = st->flags[q] & BS_FLAG_VICINITY;
            P.buffer = st->flags[q] & BS_FLAG_BUFFER;
            Cell& c = s->C(ci, cj);
            c.plist.push_back(P);
            c.ptot++;
            if (wall) c.btot++;
        }
    for (auto& c : s->cells) ensure_slots(c);
    if (gr)
        for (int q = 0; q < gr->n; ++q) {
            int ci, cj;
            if (!locate(s, gr->x[q], gr->y[q], &ci, &cj)) continue;
            s->C(ci, cj).porlist.push_back({gr->x[q], gr->y[q], gr->mass[q], gr->rho[q]});
        }
    resetid(s);
    return s;
}

void or_destroy(or_scene* s) { delete s; }
int or_n(or_scene* s) { return count_particles(s); }

void or_set_threads(int n) {
#ifdef _OPENMP
    if (n > 0) omp_set_num_threads(n);
#else
    (void)n;
#endif
}
int or_get_threads(void) {
#ifdef _OPENMP
    return omp_get_max_threads();
#else
    return 1;
#endif
}

int or_step_flags(or_scene* s, int32_t nsteps, int32_t flags) {
    if (!s || nsteps < 0 || (flags & ~BS_STEP_ALL)) return BS_E_ARG;
    for (int k = 0; k < nsteps; ++k) step(s, flags);
    return 0;
}

// bs_set_fields: overwrite particle fields in or_get's order
int or_set_fields(or_scene* s, const bs_state* st) {
    if (!s || !st || st->n != count_particles(s)) return BS_E_ARG;
    size_t q = 0;
    for (int j = 1; j <= s->cellx; ++j)
        for (int i = 1; i <= s->celly; ++i) {
            Cell& c = s->C(i, j);
            for (int k = 0; k < c.ptot; ++k, ++q) {
                Particle& p = c.plist[k];
                if (st->vx) p.vx = st->vx[q];
                if (st->vy) p.vy = st->vy[q];
                if (st->p) p.pressure = st->p[q];
                if (st->mass) p.mass = st->mass[q];
                if (st->rho) p.density = st->rho[q];
                if (st->oden) p.oden = st->oden[q];
                if (st->ovol) p.ovol = st->ovol[q];
                if (st->con) p.con = st->con[q];
            }
        }
    return 0;
}

int or_collision_shift(or_scene* s, int32_t mode, double prx, double pry, double brx, double bry) {
    if (!s || (mode != 0 && mode != 1)) return BS_E_ARG;
    collision_shift(s, mode, prx, pry, brx, bry);
    return 0;
}

int or_set_time(or_scene* s, double t) {
    if (!s) return BS_E_ARG;
    s->t = t;
    return 0;
}

int or_get(or_scene* s, bs_state* o) {
    size_t q = 0;
    for (int j = 1; j <= s->cellx; ++j)
        for (int i = 1; i <= s->celly; ++i) {
            Cell& c = s->C(i, j);
            for (int k = 0; k < c.ptot; ++k, ++q) {
                const Particle& p = c.plist[k];
                const Props& pp = c.pplist[k];
                put(o->x, q, p.x); put(o->y, q, p.y); put(o->vx, q, p.vx); put(o->vy, q, p.vy);
                put(o->p, q, p.pressure); put(o->mass, q, p.mass); put(o->rho, q, p.density);
                put(o->oden, q, p.oden); put(o->ovol, q, p.ovol); put(o->con, q, p.con);
                put(o->tid, q, (int32_t)p.tid); put(o->pid, q, (int32_t)p.pid);
                put(o->flags, q, (uint8_t)((p.free ? BS_FLAG_FREE : 0) | (p.vicinity ? BS_FLAG_VICINITY : 0) |
                                           (p.buffer ? BS_FLAG_BUFFER : 0)));
                put(o->xs, q, p.xs); put(o->ys, q, p.ys); put(o->vxs, q, p.vxs); put(o->vys, q, p.vys);
                put(o->porosity, q, pp.porosity); put(o->resx, q, pp.resistx); put(o->resy, q, pp.resisty);
                put(o->nut, q, pp.nut); put(o->tke, q, pp.tke); put(o->varts, q, pp.varts);
                put(o->gradvx, q, pp.gradvx); put(o->vel, q, pp.vel); put(o->cdiff, q, pp.cdiff);
                if (o->coff)
                    for (int r = 0; r < 4; ++r) o->coff[4 * q + r] = pp.coff[r];
                put(o->cell, q, (int32_t)s->key(i, j));
            }
        }
    return (int)q;
}

int or_info(or_scene* s, bs_scene_info* o) {
    std::memset(o, 0, sizeof(*o));
    o->n = count_particles(s);
    o->solsteps = s->solsteps;
    o->ppe_iters = s->last_iters;
    o->ppe_outer = s->last_outer;
    o->dt = s->dt;
    o->dtsol = s->dtsol;
    o->t = s->t;
    o->umax = s->umax;
    o->numax = s->numax;
    o->ppe_relres = s->last_relres;
    o->err_bits = s->err;
    return 0;
}

int or_neighbours(or_scene* s, int32_t kmax, int32_t* counts, int32_t* idx, double* dist_o, double* kx,
                  double* ky) {
    std::vector<int> start(s->cells.size() + 1, 0);
    for (size_t c = 0; c < s->cells.size(); ++c) start[c + 1] = start[c] + s->cells[c].ptot;
    size_t q = 0;
    int over = 0;
    for (size_t c = 0; c < s->cells.size(); ++c) {
        const Cell& cc = s->cells[c];
        for (int k = 0; k < cc.ptot; ++k, ++q) {
            const Verlet& L = cc.list[k];
            counts[q] = L.count;
            for (int m = 0; m < L.count; ++m) {
                if (m >= kmax) { over = 1; break; }
                size_t e = q * kmax + m;
                if (idx) idx[e] = start[L.nh[m].cell] + L.nh[m].slot;
                if (dist_o) dist_o[e] = L.dist[m];
                if (kx) kx[e] = L.kx[m];
                if (ky) ky[e] = L.ky[m];
            }
        }
    }
    return over ? BS_E_CAPACITY : 0;
}

int or_matrix(or_scene* s, int32_t kmax, double* diag, double* off, double* rhs) {
    if (!s->assembled) return BS_E_STATE;
    size_t q = 0;
    for (size_t c = 0; c < s->cells.size(); ++c) {
        const Cell& cc = s->cells[c];
        for (int k = 0; k < cc.ptot; ++k, ++q) {
            const Row& R = s->rows[cc.plist[k].matid - 1];
            if (diag) diag[q] = R.diag_total;
            if (rhs) rhs[q] = s->fvec[cc.plist[k].matid - 1];
            if (off)
                for (int m = 0; m < (int)R.off_aligned.size() && m < kmax; ++m) off[q * kmax + m] = R.off_aligned[m];
        }
    }
    return 0;
}

int or_stage(or_scene* s, int32_t stage) {
    switch (stage) {
        case OR_PROJECTION: projection(s); break;
        case OR_CELLSHIFT: cellshift(s, false); break;
        case OR_CELLSHIFTALT: cellshift(s, true); break;
        case OR_RESETID: resetid(s); break;
        case OR_NEIGHBOUR: neighbour(s); break;
        case OR_EFFPOR: effpor(s); break;
        case OR_EDDYVIS: eddyvis(s); break;
        case OR_INT_VEL: int_vel(s); break;
        case OR_PPE_ASSEMBLE: ppe_assemble(s); break;
        case OR_PPE_SOLVE: {
            int it; double rr;
            return ppe_solve(s, s->P.ppe_tol, s->P.ppe_maxit, s->P.ppe_stop, &it, &rr);
        }
        case OR_COMP_VEL: comp_vel(s); break;
        case OR_COMP_POS: comp_pos(s); break;
        case OR_FREESURF: freesurf(s); break;
        case OR_OPT2_SHIFT: opt2_shift(s); break;
        case OR_DENSITYUPDATE: densityupdate(s); break;
        case OR_TIMESTEP: timestep(s); break;
        case OR_SCALAR_SUBSTEP: scalar_substep(s); break;
        case OR_PRIME: prime(s); break;
        case OR_PRIME_SETUP: prime(s, false); break;
        case OR_CALMASSCONS: calmasscons(s); break;
        case OR_UPDATEDEN: updateden(s); break;
        case OR_DENTOPRESS: dentopress(s); break;
        case OR_PRESSTODEN: presstoden(s); break;
        case OR_WALL_PRESSURE: wall_pressure(s); break;
        case OR_EFFPOR_KEEP: effpor(s, true); break;
        case OR_BOUN_VEL: boun_vel(s); break;
        case OR_GHOST: ghost(s, false); break;
        case OR_GHOST_MLS: ghost(s, true); break;
        default: return BS_E_ARG;
    }
    return 0;
}

int or_ppe_fgmres(or_scene* s, double tol, int32_t maxit, int32_t restart, int32_t rule, int32_t* iters,
                  double* relres) {
    if (!s->assembled) return BS_E_STATE;
    if (restart < 1) return BS_E_ARG;
    const int n = s->nrows;
    s->fsol.assign(n, 0.0);   // warm start, as ppe_solve
    for (auto& c : s->cells)
        for (int k = 0; k < c.ptot; ++k) s->fsol[c.plist[k].matid - 1] = c.plist[k].pressure;
    int it = 0;
    double rr = 0;
    const int st = fgmres(
        n, [&](const std::vector<double>& b, std::vector<double>& r) { spmv2(s, b, r); }, s->fvec, s->fsol, tol,
        maxit, restart, rule, &it, &rr);
    for_interior(s, [&](int i, int j) {
        Cell& c = s->C(i, j);
        for (int k = 0; k < c.ptot; ++k) c.plist[k].pressure = s->fsol[c.plist[k].matid - 1];
    });
    s->last_iters = it;
    s->last_relres = rr;
    if (st) s->err |= BS_ERR_NOT_CONVERGED;
    if (iters) *iters = it;
    if (relres) *relres = rr;
    return st ? BS_E_NOTCONV : 0;
}

int or_fgmres_csr(int32_t n, const int32_t* row_ptr, const int32_t* col, const double* val, const double* b,
                  double* x, double tol, int32_t maxit, int32_t restart, int32_t rule, int32_t* iters,
                  double* relres) {
    if (n <= 0 || restart < 1) return BS_E_ARG;
    auto spmv = [&](const std::vector<double>& v, std::vector<double>& r) {
        for (int is = 0; is < n; ++is) {
            double comp = 0.0;
            for (int js = row_ptr[is]; js < row_ptr[is + 1]; ++js) comp = comp + val[js] * v[col[js]];
            r[is] = comp;
        }
    };
    std::vector<double> bb(b, b + n), sl(x, x + n);
    int it = 0;
    double rr = 0;
    const int st = fgmres(n, spmv, bb, sl, tol, maxit, restart, rule, &it, &rr);
    for (int k = 0; k < n; ++k) x[k] = sl[k];
    if (iters) *iters = it;
    if (relres) *relres = rr;
    return st ? BS_E_NOTCONV : 0;
}

int or_ppe_solve(or_scene* s, double tol, int32_t maxit, int32_t rule, int32_t* iters, double* relres) {
    if (!s->assembled) return BS_E_STATE;
    int it = 0;
    double rr = 0;
    int st = ppe_solve(s, tol, maxit, rule, &it, &rr);
    if (iters) *iters = it;
    if (relres) *relres = rr;
    return st ? BS_E_NOTCONV : 0;
}

int or_step(or_scene* s, int32_t nsteps) {
    for (int k = 0; k < nsteps; ++k) step(s);
    return 0;
}

// combined, output.f90:188-222 (gfortran's Fw.d / ESw.d: right justified,
// asterisks when the value does not fit)
static void ffmt(std::string& o, double v, int w, int d, bool es) {
    char b[64];
    std::snprintf(b, sizeof b, es ? "%*.*E" : "%*.*f", w, d, v);
    o += (int)std::strlen(b) > w ? std::string(w, '*') : std::string(b);
}
int or_write_combined(or_scene* s, const char* fluid_path, const char* buffer_path) {
    FILE* ff = std::fopen(fluid_path, "w");
    if (!ff) return BS_E_ARG;
    FILE* fb = buffer_path ? std::fopen(buffer_path, "w") : nullptr;
    for (int j = 2; j <= s->cellx - 1; ++j)
        for (int i = 2; i <= s->celly - 1; ++i) {
            const Cell& c = s->C(i, j);
            for (int k = 0; k < c.ptot; ++k) {
                const Particle& p = c.plist[k];
                if (p.tid != 3) continue;
                FILE* f = p.buffer ? fb : ff;
                if (!f) continue;
                std::string o;
                ffmt(o, p.x, 10, 3, false); o += ' ';
                ffmt(o, p.y, 10, 3, false); o += ' ';
                ffmt(o, p.pressure, 10, 3, false); o += ' ';
                ffmt(o, p.vx, 10, 3, true); o += ' ';
                ffmt(o, p.vy, 10, 3, true); o += ' ';
                ffmt(o, p.con + 0.50, 10, 5, false);
                o += '\n';
                std::fputs(o.c_str(), f);
            }
        }
    std::fclose(ff);
    if (fb) std::fclose(fb);
    return 0;
}

int or_wcsph_step(or_scene* s, int32_t nsteps) {
    for (int k = 0; k < nsteps; ++k) wcsph_step(s);
    return 0;
}

int or_set_inflow(or_scene* s, int32_t zone, const bs_inflow* z) {
    if (!s || zone < 0 || zone > 1 || !z || z->n < 0 || z->ncells < 0) return BS_E_ARG;
    OrZone Z;
    if (z->n == 0 && z->ncells == 0) {
        s->zones[zone] = Z;
        return 0;
    }
    if ((z->n && (!z->x || !z->y || !z->vx || !z->vy || !z->p)) || (z->ncells && (!z->cell_i || !z->cell_j)) ||
        (z->remove_side != 1 && z->remove_side != -1) || !(z->rho > 0))
        return BS_E_ARG;
    for (int q = 0; q < z->ncells; ++q) {
        const int i = z->cell_i[q], j = z->cell_j[q];
        if (i < 2 || i > s->celly - 1 || j < 2 || j > s->cellx - 1) return BS_E_ARG;
        for (int u = 0; u < q; ++u)
            if (z->cell_i[u] == i && z->cell_j[u] == j) return BS_E_ARG;
        Z.cells.push_back({i, j});
    }
    for (int q = 0; q < z->n; ++q) {   // bufferN(k,i) with insert_bufferN's assignments
        Particle t;
        t.x = z->x[q];
        t.y = z->y[q];
        t.vx = z->vx[q];
        t.vy = z->vy[q];
        t.pressure = z->p[q];
        t.pid = z->pid ? z->pid[q] : 0;
        t.tid = 3;
        t.buffer = true;
        t.mass = z->mass;
        t.density = z->rho;
        t.oden = z->rho;
        t.ovol = z->ovol;
        t.con = z->con;
        Z.tmpl.push_back(t);
    }
    Z.period = z->period;
    Z.phase = z->phase;
    Z.remove_x = z->remove_x;
    Z.side = z->remove_side;
    Z.set = true;
    s->zones[zone] = Z;
    return 0;
}

int or_buffer_exchange(or_scene* s, int32_t zone) {
    if (!s || zone < 0 || zone > 1 || !s->zones[zone].set) return BS_E_ARG;
    buffer_exchange(s, zone);
    return 0;
}

int or_set_pressure(or_scene* s, const double* p) {
    size_t q = 0;
    for (auto& c : s->cells)
        for (int k = 0; k < c.ptot; ++k, ++q) c.plist[k].pressure = p[q];
    return 0;
}

int or_bicgstab_csr(int32_t n, const int32_t* row_ptr, const int32_t* col, const double* val, const double* b,
                    double* x, double tol, int32_t maxit, int32_t rule, int32_t* iters, double* relres) {
    // CSR operator spmv, solver.f90:53-82 (0-based here)
    auto spmv = [&](const std::vector<double>& v, std::vector<double>& r) {
        for (int is = 0; is < n; ++is) {
            double comp = 0.0;
            for (int js = row_ptr[is]; js < row_ptr[is + 1]; ++js) comp = comp + val[js] * v[col[js]];
            r[is] = comp;
        }
    };
    std::vector<double> bb(b, b + n), sl(x, x + n);
    int it = 0;
    double rr = 0;
    int st = bicgstab(n, spmv, bb, sl, tol, maxit, rule, &it, &rr);
    for (int k = 0; k < n; ++k) x[k] = sl[k];
    if (iters) *iters = it;
    if (relres) *relres = rr;
    return st ? BS_E_NOTCONV : 0;
}

double or_Wab(double r, double h) { return Wab(r, h); }
double or_Wo(double h) { return Wo(h); }
void or_gradW(double xj, double yj, double xi, double yi, double r, double h, double* wx, double* wy) {
    *wx = Wgrad(xi - xj, r, h);
    *wy = Wgrad(yi - yj, r, h);
}
void or_invert2(double* a4) { invertmat2D(a4); }
double or_vis(double oden) { return vis(oden); }

}  // extern "C"
