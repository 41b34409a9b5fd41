// TEST INFRASTRUCTURE ONLY: driver of the reference translated by
// oracle/ref_translate.py (compiled by oracle/ref_build.py with the
// generated modules force-included).  It runs the reference's own main
// program, main.f90:23-272, with the three loops cut to the given step
// counts: the set-up (init, gen_boundary, gen_fluid, memalloc, matrixid,
// effpor), the first settling phase, the fluid put at rest, the settling
// phase with the open-boundary buffers, the salinity set-up and time reset,
// and the production steps with the salinity sub-steps, the density update
// and the closing eddyvis.  The writers of output.f90 are not called; the
// driver writes the particle state instead.
//
//     ref_main <out prefix> <settle steps> <buffer steps> <production steps> [dump every
//              [ins_1 ins_2]]
//
// ins_1, ins_2 (optional) replace the exchange periods of the two buffer
// zones that gen_fluid sets (internal.f90), so that short runs exchange.
//
// Dumps <prefix>_<global step>.bin after the set-up (0), every `dump every`
// steps and at the end of each phase: int64 count, then per particle (cells
// in the reference's column-major order, sx..ex x sy..ey, slots 1..ptot) REC
// doubles: pid, tid, x, y, vx, vy, pressure, density, mass, con, oden, ovol,
// buffer, free, porosity, nut, tke, cell j, cell i, slot, dt, t.
#include <cstdio>
#include <cstdlib>
#include <vector>

static const int REC = 22;

static void dump(const char* prefix, int step) {
    char path[4096];
    std::snprintf(path, sizeof path, "%s_%d.bin", prefix, step);
    std::vector<double> rec;
    auto& C = initialize__dpcell;
    for (int j = initialize__sx; j <= initialize__ex; ++j)
        for (int i = initialize__sy; i <= initialize__ey; ++i) {
            T_cell& c = C(i, j);
            for (int k = 1; k <= c.ptot_; ++k) {
                const T_particles& p = c.plist_(k);
                const T_properties& q = c.pplist_(k);
                const double v[REC] = {(double)p.pid_, (double)p.tid_, p.x_, p.y_, p.vx_, p.vy_, p.pressure_,
                                       p.density_, p.mass_, p.con_, p.oden_, p.ovol_, (double)p.buffer_,
                                       (double)p.free_, q.porosity_, q.nut_, q.tke_, (double)j, (double)i,
                                       (double)k, initialize__dt, initialize__t};
                rec.insert(rec.end(), v, v + REC);
            }
        }
    FILE* f = std::fopen(path, "wb");
    if (!f) {
        std::perror(path);
        std::exit(2);
    }
    const long long n = (long long)(rec.size() / REC);
    std::fwrite(&n, sizeof n, 1, f);
    std::fwrite(rec.data(), sizeof(double), rec.size(), f);
    std::fclose(f);
}

static void step_stages(bool production) {
    isph__projection();
    integrator__cellshift();
    isph__resetid();
    search__neighbour();
    porous__effpor();
    turbulence__eddyvis();
    integrator__int_vel();
    isph__ppesolve();
    integrator__comp_vel();
    integrator__comp_pos();
    integrator__cellshiftalt();
    search__neighbour();
    isph__freesurf();
    porous__effpor();
    part_shift__opt2_shift();
    if (production) scalar__densityupdate();
    integrator__timestep();
    if (production) turbulence__eddyvis();
}

int main(int argc, char** argv) {
    if (argc < 5) {
        std::fprintf(stderr, "usage: %s <out prefix> <settle> <buffer settle> <production> [dump every]\n", argv[0]);
        return 1;
    }
    const char* prefix = argv[1];
    const int n1 = std::atoi(argv[2]), n2 = std::atoi(argv[3]), n3 = std::atoi(argv[4]);
    const int every = argc > 5 ? std::atoi(argv[5]) : 1 << 30;
    int g = 0;   // global step count (dump label)
    // main.f90:23-37
    setup__init();
    boundary__gen_boundary();
    internal__gen_fluid();
    memory__memalloc();
    if (argc > 7) {
        initialize__ins_1 = std::atof(argv[6]);
        initialize__ins_2 = std::atof(argv[7]);
    }
    memory__matrixid();
    initialize__iter = initialize__iter + 1;
    porous__effpor();
    dump(prefix, 0);
    // main.f90:39-64: settling without buffers and salinity
    for (int s = 1; s <= n1; ++s) {
        initialize__told = initialize__t;
        initialize__t = initialize__t + initialize__dt;
        step_stages(false);
        initialize__iter = initialize__iter + 1;
        ++g;
        if (g % every == 0 || s == n1) dump(prefix, g);
    }
    // main.f90:66-92: the fluid at rest
    initialize__iter = 1;
    auto& C = initialize__dpcell;
    for (int j = initialize__sx; j <= initialize__ex; ++j)
        for (int i = initialize__sy; i <= initialize__ey; ++i) {
            T_cell& c = C(i, j);
            for (int k = 1; k <= c.ptot_; ++k) {
                T_particles& p = c.plist_(k);
                if (p.tid_ == 3 && !p.buffer_) {
                    p.vx_ = 0.0;
                    p.vy_ = 0.0;
                }
            }
        }
    initialize__iter1 = 1;
    initialize__iter2 = 1;
    // main.f90:94-147: settling with the buffers (the open side at relative density 1)
    double one = 1.0;
    for (int s = 1; s <= n2; ++s) {
        initialize__told = initialize__t;
        initialize__t = initialize__t + initialize__dt;
        if (initialize__told < initialize__iter1 * initialize__ins_1 &&
            initialize__t >= initialize__iter1 * initialize__ins_1) {
            internal__remove_buffer1();
            internal__insert_buffer1();
            initialize__iter1 = initialize__iter1 + 1;
        }
        if (initialize__told < initialize__iter2 * initialize__ins_2 &&
            initialize__t >= initialize__iter2 * initialize__ins_2) {
            internal__remove_buffer2();
            internal__insert_buffer2(one);
            initialize__iter2 = initialize__iter2 + 1;
        }
        step_stages(false);
        initialize__iter = initialize__iter + 1;
        ++g;
        if (g % every == 0 || s == n2) dump(prefix, g);
    }
    // main.f90:149-197: salt water above the coast line; t restarts at 0
    for (int j = initialize__sx; j <= initialize__ex; ++j)
        for (int i = initialize__sy; i <= initialize__ey; ++i) {
            T_cell& c = C(i, j);
            for (int k = 1; k <= c.ptot_; ++k) {
                T_particles& p = c.plist_(k);
                if (p.tid_ == 3) {
                    p.con_ = -0.50;
                    if (((p.y_ - initialize__yl) - initialize__line_grad * (p.x_ - initialize__xl)) > 0.0f) {
                        p.mass_ = p.mass_ * initialize__rel_den;
                        p.oden_ = p.oden_ * initialize__rel_den;
                        p.density_ = p.density_ * initialize__rel_den;
                        p.con_ = 0.50;
                    }
                }
            }
        }
    initialize__time_shift = initialize__t;
    initialize__iter = 1;
    initialize__iter1 = 1;
    initialize__iter2 = 1;
    initialize__t = 0.0;
    // main.f90:199-272: production
    for (int s = 1; s <= n3; ++s) {
        initialize__told = initialize__t;
        initialize__t = initialize__t + initialize__dt;
        for (int j1 = 1; j1 <= initialize__solsteps; ++j1) {
            scalar__scalart_anisotropic();
            scalar__scalarupdate(initialize__dtsol);
        }
        if ((initialize__told + initialize__time_shift) < initialize__iter1 * initialize__ins_1 &&
            (initialize__t + initialize__time_shift) >= initialize__iter1 * initialize__ins_1) {
            internal__remove_buffer1();
            internal__insert_buffer1();
            initialize__iter1 = initialize__iter1 + 1;
        }
        if ((initialize__told + initialize__time_shift) < initialize__iter2 * initialize__ins_2 &&
            (initialize__t + initialize__time_shift) >= initialize__iter2 * initialize__ins_2) {
            internal__remove_buffer2();
            internal__insert_buffer2(initialize__rel_den);
            initialize__iter2 = initialize__iter2 + 1;
        }
        step_stages(true);
        ++g;
        if (g % every == 0 || s == n3) dump(prefix, g);
    }
    return 0;
}
