// main.cpp -- nbody_gb300: the deck-driven batch front end.
//
// The headless subset of projects/02_nbody_gravity/src/main.cpp:
//   nbody_gb300 --deck <f.toml> --out <dir> [--frames N] [--substeps N]
//   nbody_gb300 --bench <solver> [--bench-n N] [--bench-theta T] [--bench-reps R] [--bench-eps E]
//   nbody_gb300 --dump-ic <file.bin> [--bench-n N]
//   nbody_gb300 --deck <f.toml> --dump-ic <file.bin>   (the deck's scenario; no GPU)
//   nbody_gb300 --selftest | --rung-selftest | --dt-selftest
//   nbody_gb300 --print-deck <f.toml>        (parsed deck as JSON; no GPU)
// Flags as in main.cpp:35-95; --bench prints the same CSV line
// (main.cpp:389-391), --dump-ic writes the same raw float32 records
// (main.cpp:253-280).  GL modes (--interactive, --render-check,
// --gpu-selftest) do not exist here: there is no graphics stack.
#include "deck.hpp"
#include "deck_sim.hpp"
#include "ngrav_gpu.h"
#include "scenarios.hpp"
#include "simulation.hpp"

#include <algorithm>
#include <chrono>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <stdexcept>
#include <string>
#include <vector>

namespace {

struct Args {
    std::string deck, out, bench, dumpIc, printDeck;
    int frames = 0, substeps = 0;
    bool selftest = false, rungSelftest = false, dtSelftest = false;
    int benchN = 10000;
    double benchTheta = 0.5;
    int benchReps = 5;
    int benchOrder = 5;
    double benchEps = 0.02;
    int leafCapacity = 8;
};

Args ParseArgs(int argc, char** argv) {
    Args a;
    for (int i = 1; i < argc; ++i) {
        const std::string s = argv[i];
        auto next = [&]() { return (i + 1 < argc) ? argv[++i] : ""; };
        if (s == "--deck") a.deck = next();
        else if (s == "--out") a.out = next();
        else if (s == "--frames") a.frames = std::atoi(next());
        else if (s == "--substeps") a.substeps = std::atoi(next());
        else if (s == "--selftest") a.selftest = true;
        else if (s == "--rung-selftest") a.rungSelftest = true;
        else if (s == "--dt-selftest") a.dtSelftest = true;
        else if (s == "--bench") a.bench = next();
        else if (s == "--bench-n") a.benchN = std::atoi(next());
        else if (s == "--bench-theta") a.benchTheta = std::atof(next());
        else if (s == "--bench-reps") a.benchReps = std::atoi(next());
        else if (s == "--bench-order") a.benchOrder = std::atoi(next());
        else if (s == "--bench-eps") a.benchEps = std::atof(next());
        else if (s == "--leaf-capacity") a.leafCapacity = std::atoi(next());
        else if (s == "--dump-ic") a.dumpIc = next();
        else if (s == "--print-deck") a.printDeck = next();
        else std::fprintf(stderr, "warning: unknown arg '%s'\n", s.c_str());
    }
    return a;
}

void Check(int rc, ngrav_gpu_ctx* ctx, const char* what) {
    if (rc != NGRAV_OK) {
        std::fprintf(stderr, "%s failed (%d): %s\n", what, rc, ctx ? ngrav_gpu_last_error(ctx) : "");
        std::exit(1);
    }
}

ngrav_gpu_ctx* MakeContext(double G, double eps, double theta, int leafCap) {
    ngrav_gpu_opts o;
    ngrav_gpu_default_opts(&o);
    o.G = G;
    o.eps = eps;
    o.theta = theta;
    o.leaf_capacity = leafCap;
    ngrav_gpu_ctx* ctx = nullptr;
    Check(ngrav_gpu_create(&ctx, &o), nullptr, "ngrav_gpu_create");
    return ctx;
}

// --bench (main.cpp:287-393): mean per-evaluation wall time of one force
// evaluation (host arrays in, accelerations out) on the Plummer sphere the
// reference benches (seed 1), and the mean relative error against the
// exact sum for N <= 60000 (-1 otherwise).
int RunBench(const Args& a) {
    const bool direct = a.bench == "direct" || a.bench == "gpu_direct";
    const bool bh = a.bench == "barnes_hut" || a.bench == "bh" || a.bench == "gpu_bh" || a.bench == "gpu_barnes_hut";
    if (!direct && !bh) {
        std::fprintf(stderr, "bench: unknown solver '%s' (barnes_hut|bh|gpu_bh|direct|gpu_direct)\n", a.bench.c_str());
        return 2;
    }
    const ngrav_host::State s = ngrav_host::Plummer(a.benchN, 1);
    const double theta = direct ? 0.0 : a.benchTheta;
    ngrav_gpu_ctx* ctx = MakeContext(1.0, a.benchEps, theta, a.leafCapacity);
    const size_t n = s.Count();
    std::vector<double> ax(n), ay(n), az(n);
    auto eval = [&]() {
        Check(ngrav_gpu_set_particles(ctx, (int64_t)n, s.x.data(), s.y.data(), s.z.data(), nullptr, nullptr,
                                      nullptr, s.m.data()),
              ctx, "set_particles");
        Check(ngrav_gpu_compute_accel(ctx, ax.data(), ay.data(), az.data()), ctx, "compute_accel");
    };
    eval();  // warm
    const auto t0 = std::chrono::steady_clock::now();
    for (int r = 0; r < a.benchReps; ++r) eval();
    const auto t1 = std::chrono::steady_clock::now();
    const double ms = std::chrono::duration<double, std::milli>(t1 - t0).count() / a.benchReps;
    double meanRel = -1.0;
    if (a.benchN <= 60000) {
        ngrav_gpu_ferr fe;
        Check(ngrav_gpu_force_error(ctx, (int)n, 1, 1, &fe), ctx, "force_error");
        meanRel = fe.mean;
    }
    ngrav_gpu_destroy(ctx);
    std::fprintf(stderr, "solver,n,theta,order,ms_per_eval,mean_rel_err\n");
    std::printf("%s,%d,%.3f,%d,%.4f,%.6e\n", a.bench.c_str(), a.benchN, a.benchTheta, a.benchOrder, ms, meanRel);
    return 0;
}

int DumpIc(const Args& a) {
    const ngrav_host::State s = ngrav_host::Plummer(a.benchN, 1);
    ngrav_host::WriteIcFile(a.dumpIc, s);
    std::fprintf(stderr, "# dump-ic path=%s N=%d eps=%.5g G=%.4f seed=%u format=raw-f32-x,y,z,m,vx,vy,vz\n",
                 a.dumpIc.c_str(), a.benchN, a.benchEps, 1.0, 1u);
    return 0;
}

// --deck <f.toml> --dump-ic <file.bin>: the deck's scenario in the same raw
// format, with the scenario's G / softening / dt on stderr.  Needs no GPU.
int DumpDeckIc(const Args& a) {
    const fw::Deck deck = fw::Deck::FromFile(a.deck);
    ngrav_host::ScenarioParams p;
    p.n = deck.GetInt("scenario.n", 2000);
    p.seed = (uint32_t)deck.GetInt("scenario.seed", 1);
    p.icFile = deck.GetString("scenario.ic_file", "");
    const std::string type = deck.GetString("scenario.type", "plummer");
    bool fellBack = false;
    const ngrav_host::Scenario sc = ngrav_host::BuildScenario(type, p, &fellBack);
    if (fellBack) std::fprintf(stderr, "warning: scenario.type = \"%s\" is not available; Plummer used\n", type.c_str());
    ngrav_host::WriteIcFile(a.dumpIc, sc.state);
    std::fprintf(stderr, "# scenario type=%s N=%zu G=%.17g eps=%.17g dt=%.17g\n", type.c_str(), sc.state.Count(),
                 sc.G, sc.eps, sc.suggestedDt);
    return 0;
}

void CheckPrint(bool& ok, const char* name, double value, double tol) {
    const bool good = std::isfinite(value) && std::abs(value) <= tol;
    std::printf("  %-44s %12.4e  (tol %.1e)  %s\n", name, value, tol, good ? "ok" : "WRONG");
    if (!good) ok = false;
}

double Energy(ngrav_gpu_ctx* ctx) {
    ngrav_gpu_diag d;
    Check(ngrav_gpu_diagnostics(ctx, 1, &d), ctx, "diagnostics");
    return d.energy;
}

long long StatsField(ngrav_gpu_ctx* ctx, long long ngrav_gpu_stats::*f) {
    ngrav_gpu_stats st;
    Check(ngrav_gpu_get_stats(ctx, &st), ctx, "get_stats");
    return st.*f;
}

// Integrate an n-body set with exact pair sums (theta = 0) for `steps` KDK
// steps; `each(ctx, k)` runs after every step.
template <class F>
void RunExact(const std::vector<double>& x, const std::vector<double>& y, const std::vector<double>& vx,
              const std::vector<double>& vy, const std::vector<double>& m, double eps, bool spline, double dt,
              int steps, F each) {
    const size_t n = m.size();
    std::vector<double> z(n, 0.0), vz(n, 0.0);
    ngrav_gpu_ctx* ctx = MakeContext(1.0, eps, 0.0, 8);
    if (spline) Check(ngrav_gpu_set_softening(ctx, NGRAV_SOFTENING_SPLINE), ctx, "set_softening");
    Check(ngrav_gpu_set_particles(ctx, (int64_t)n, x.data(), y.data(), z.data(), vx.data(), vy.data(), vz.data(),
                                  m.data()),
          ctx, "set_particles");
    Check(ngrav_gpu_prime(ctx), ctx, "prime");
    each(ctx, -1);
    for (int k = 0; k < steps; ++k) {
        Check(ngrav_gpu_step(ctx, 1, dt), ctx, "step");
        each(ctx, k);
    }
    ngrav_gpu_destroy(ctx);
}

struct Range {
    double lo = 1e300, hi = -1e300;
    void Add(double v) {
        lo = std::min(lo, v);
        hi = std::max(hi, v);
    }
    double Drift() const { return (hi - lo) / std::abs(0.5 * (hi + lo)); }
};

std::vector<double> Positions(ngrav_gpu_ctx* ctx, size_t n) {
    std::vector<double> s(6 * n);
    Check(ngrav_gpu_get_state(ctx, s.data(), s.data() + n, s.data() + 2 * n, s.data() + 3 * n, s.data() + 4 * n,
                              s.data() + 5 * n),
          ctx, "get_state");
    return s;
}

double HalfMassRadius(const std::vector<double>& st, size_t n) {
    std::vector<double> r(n);
    for (size_t i = 0; i < n; ++i) r[i] = std::sqrt(st[i] * st[i] + st[n + i] * st[n + i] + st[2 * n + i] * st[2 * n + i]);
    std::sort(r.begin(), r.end());
    return r[n / 2];
}

// The self-test gates of the reference (CoreSelfTest3D, SelfTest.cpp:78-265,
// and the Plummer part of CoreIcSelfTest, :729-777) on the GPU path.  Force
// arithmetic is FP32 with double-float positions and velocities, so the
// gates that ask for FP64 round-off (1e-12 force equalities, the triangle's
// 2e-8 energy drift) take FP32 tolerances, marked as such, and the
// Lagrange triangle is reported without a gate.
int SelfTest() {
    bool ok = true;
    const double kPi = 3.14159265358979323846;
    {
        std::printf("[kepler 3D, GPU]\n");
        const double sep = 1.0, vRel = 0.8 * std::sqrt(2.0 / sep);
        const double period = 2.0 * kPi * std::sqrt(sep * sep * sep / 2.0);
        double rMin = 1e30, rMax = 0.0;
        Range E, L;
        RunExact({-sep / 2, sep / 2}, {0, 0}, {0, 0}, {-vRel / 2, vRel / 2}, {1.0, 1.0}, 1e-6, false, period / 2000.0,
                 4 * 2000, [&](ngrav_gpu_ctx* ctx, int k) {
                     if (k >= 0) {
                         const std::vector<double> st = Positions(ctx, 2);
                         const double r = std::hypot(st[1] - st[0], st[3] - st[2], st[5] - st[4]);
                         rMin = std::min(rMin, r);
                         rMax = std::max(rMax, r);
                     }
                     if (k < 0 || k % 50 == 0) {
                         ngrav_gpu_diag d;
                         Check(ngrav_gpu_diagnostics(ctx, 1, &d), ctx, "diagnostics");
                         E.Add(d.energy);
                         L.Add(std::sqrt(d.L[0] * d.L[0] + d.L[1] * d.L[1] + d.L[2] * d.L[2]));
                     }
                 });
        const double a = 1.0 / 1.36;
        CheckPrint(ok, "periapsis rel err", (rMin - a * (1.0 - 0.36)) / (a * (1.0 - 0.36)), 1e-4);
        CheckPrint(ok, "apoapsis rel err", rMax - 1.0, 1e-4);
        CheckPrint(ok, "energy drift", E.Drift(), 1e-4);
        CheckPrint(ok, "|L| drift", L.Drift(), 1e-6);
    }
    {
        std::printf("[lagrange triangle 3D, GPU]\n");
        const double Ls = 1.0, omega = std::sqrt(3.0 / (Ls * Ls * Ls)), R = Ls / std::sqrt(3.0);
        std::vector<double> x(3), y(3), vx(3), vy(3);
        for (int k = 0; k < 3; ++k) {
            const double ang = 2.0 * kPi * k / 3.0;
            x[k] = R * std::cos(ang);
            y[k] = R * std::sin(ang);
            vx[k] = -omega * R * std::sin(ang);
            vy[k] = omega * R * std::cos(ang);
        }
        double shape = 0.0;
        Range E;
        RunExact(x, y, vx, vy, {1.0, 1.0, 1.0}, 1e-6, false, (2.0 * kPi / omega) / 2000.0, 5 * 2000,
                 [&](ngrav_gpu_ctx* ctx, int k) {
                     if (k >= 0) {
                         const std::vector<double> st = Positions(ctx, 3);
                         for (int a = 0; a < 3; ++a) {
                             const int b = (a + 1) % 3;
                             const double d = std::hypot(st[b] - st[a], st[3 + b] - st[3 + a], st[6 + b] - st[6 + a]);
                             shape = std::max(shape, std::abs(d - Ls) / Ls);
                         }
                     }
                     if (k < 0 || k % 50 == 0) E.Add(Energy(ctx));
                 });
        // Not a gate here: the equal-mass triangle is a linearly unstable
        // equilibrium, and FP32 force round-off (~1e-7) grows past the
        // reference's 1e-5 shape bound within the five periods (FP64
        // round-off, 1e-16, does not).
        std::printf("  triangle shape deviation %.4e, energy drift %.4e  (informational: unstable equilibrium, FP32 "
                    "forces)\n",
                    shape, E.Drift());
    }
    {
        std::printf("[spline softening 3D, GPU]\n");
        const double h = 0.1;
        double maxRel = 0.0;
        uint64_t st = 777;
        for (int t = 0; t < 200; ++t) {
            st = st * 6364136223846793005ull + 1442695040888963407ull;
            const double r = 2.0 * h + 3.0 * h * (double)(st >> 11) / 9007199254740992.0;
            const double x[2] = {0.0, r}, zero[2] = {0.0, 0.0}, mm[2] = {1.0, 1.0};
            ngrav_gpu_ctx* ctx = MakeContext(1.0, h, 0.0, 8);
            Check(ngrav_gpu_set_softening(ctx, NGRAV_SOFTENING_SPLINE), ctx, "set_softening");
            Check(ngrav_gpu_set_particles(ctx, 2, x, zero, zero, zero, zero, zero, mm), ctx, "set_particles");
            double ax[2], ay[2], az[2];
            Check(ngrav_gpu_compute_accel(ctx, ax, ay, az), ctx, "compute_accel");
            ngrav_gpu_destroy(ctx);
            const double exact = 1.0 / (r * r);
            maxRel = std::max(maxRel, std::abs(ax[0] - exact) / exact);
        }
        CheckPrint(ok, "spline force == Newtonian for r>=2h (FP32; reference 1e-12)", maxRel, 1e-6);
        const double sep = 1.0, e = 0.5;
        const double vRel = std::sqrt(2.0 * (2.0 / sep - (1.0 + e) / sep));
        const double a = sep / (1.0 + e);
        const double period = 2.0 * kPi * std::sqrt(a * a * a / 2.0);
        Range E;
        RunExact({-sep / 2, sep / 2}, {0, 0}, {0, 0}, {-vRel / 2, vRel / 2}, {1.0, 1.0}, 0.02, true, period / 3000.0,
                 4 * 3000, [&](ngrav_gpu_ctx* ctx, int k) {
                     if (k < 0 || k % 50 == 0) E.Add(Energy(ctx));
                 });
        CheckPrint(ok, "spline-softened orbit energy drift", E.Drift(), 1e-4);
    }
    {
        std::printf("[plummer IC, GPU]\n");
        const ngrav_host::State s = ngrav_host::Plummer(20000, 3);
        const size_t n = s.Count();
        ngrav_gpu_ctx* ctx = MakeContext(1.0, 0.05, 0.5, 8);  // eps^2 = 0.0025 as VirialRatio
        Check(ngrav_gpu_set_particles(ctx, (int64_t)n, s.x.data(), s.y.data(), s.z.data(), s.vx.data(), s.vy.data(),
                                      s.vz.data(), s.m.data()),
              ctx, "set_particles");
        ngrav_gpu_diag d;
        Check(ngrav_gpu_diagnostics(ctx, 1, &d), ctx, "diagnostics");
        ngrav_gpu_destroy(ctx);
        const double vr = 2.0 * d.kinetic / std::abs(d.potential);
        std::printf("  Plummer  2T/|W| = %.3f\n", vr);
        CheckPrint(ok, "Plummer virial ratio |2T/|W| - 1|", vr - 1.0, 0.12);
        // dynamical hold: 2,000 bodies, Barnes-Hut theta 0.5, ~6 crossing times
        const ngrav_host::State s2 = ngrav_host::Plummer(2000, 5);
        const size_t n2 = s2.Count();
        ngrav_gpu_ctx* c2 = MakeContext(1.0, 0.05, 0.5, 8);
        Check(ngrav_gpu_set_particles(c2, (int64_t)n2, s2.x.data(), s2.y.data(), s2.z.data(), s2.vx.data(),
                                      s2.vy.data(), s2.vz.data(), s2.m.data()),
              c2, "set_particles");
        const double rh0 = HalfMassRadius(Positions(c2, n2), n2);
        const double dt = (2.0 * kPi) / 400.0;
        Check(ngrav_gpu_prime(c2), c2, "prime");
        Check(ngrav_gpu_step(c2, (int)(6.0 * (2.0 * kPi) / dt), dt), c2, "step");
        const double rh1 = HalfMassRadius(Positions(c2, n2), n2);
        ngrav_gpu_destroy(c2);
        const double drift = std::abs(rh1 - rh0) / rh0;
        std::printf("  Plummer  half-mass radius: %.4f -> %.4f over ~6 t_cross (drift %.1f%%)\n", rh0, rh1,
                    100.0 * drift);
        CheckPrint(ok, "Plummer half-mass radius drift over ~6 t_cross", drift, 0.15);
    }
    {
        std::printf("[barnes-hut vs direct 3D, GPU]\n");
        const ngrav_host::State s = ngrav_host::UniformCubeCloud(1000, 12345);
        const size_t n = s.Count();
        ngrav_gpu_ctx* ctx = MakeContext(1.0, 0.02, 0.0, 8);
        Check(ngrav_gpu_set_particles(ctx, (int64_t)n, s.x.data(), s.y.data(), s.z.data(), nullptr, nullptr, nullptr,
                                      s.m.data()),
              ctx, "set_particles");
        std::vector<double> ax(n), ay(n), az(n);
        Check(ngrav_gpu_compute_accel(ctx, ax.data(), ay.data(), az.data()), ctx, "compute_accel");
        ngrav_gpu_ferr fe;
        Check(ngrav_gpu_force_error(ctx, (int)n, 1, 1, &fe), ctx, "force_error");
        CheckPrint(ok, "max per-particle |da|/|a| (theta=0, FP32)", fe.max, 1e-5);
        ngrav_gpu_destroy(ctx);
    }
    {
        std::printf("[quadrupole barnes-hut 3D, GPU]\n");
        const ngrav_host::State s = ngrav_host::UniformBallCloud(4000, 2024);
        const size_t n = s.Count();
        double err[2];
        for (int q = 0; q < 2; ++q) {
            ngrav_gpu_opts o;
            ngrav_gpu_default_opts(&o);
            o.G = 1.0;
            o.eps = 0.01;
            o.theta = 0.5;
            o.quadrupole = q;
            ngrav_gpu_ctx* ctx = nullptr;
            Check(ngrav_gpu_create(&ctx, &o), nullptr, "create");
            Check(ngrav_gpu_set_particles(ctx, (int64_t)n, s.x.data(), s.y.data(), s.z.data(), nullptr, nullptr,
                                          nullptr, s.m.data()),
                  ctx, "set_particles");
            std::vector<double> ax(n), ay(n), az(n);
            Check(ngrav_gpu_compute_accel(ctx, ax.data(), ay.data(), az.data()), ctx, "compute_accel");
            ngrav_gpu_ferr fe;
            Check(ngrav_gpu_force_error(ctx, (int)n, 1, 1, &fe), ctx, "force_error");
            err[q] = fe.max;
            ngrav_gpu_destroy(ctx);
        }
        std::printf("  theta=0.5: monopole-only max err=%.3e   mono+quad max err=%.3e   improvement=%.2fx\n", err[0],
                    err[1], err[0] / std::max(err[1], 1e-30));
        CheckPrint(ok, "quadrupole gives >=3x lower max force err", std::max(0.0, 3.0 - err[0] / err[1]), 0.0);
    }
    std::printf("\nselftest: %s\n", ok ? "PASS" : "FAIL");
    return ok ? 0 : 1;
}

// CoreRungSelfTest (SelfTest.cpp:821-924) on the GPU path: a 200-body cloud
// plus a tight binary under the block, global-adaptive and fixed schemes
// (exact pair sums, theta = 0), and a Barnes-Hut cold collapse under the
// block scheme.
int RungSelfTest() {
    bool ok = true;
    std::printf("[block / rung timesteps, GPU]\n");
    {
        ngrav_host::State cloud = ngrav_host::Plummer(200, 12);
        ngrav_host::State s;
        const int n = 202;
        s.x.assign(n, 0.0); s.y.assign(n, 0.0); s.z.assign(n, 0.0);
        s.vx.assign(n, 0.0); s.vy.assign(n, 0.0); s.vz.assign(n, 0.0); s.m.assign(n, 0.0);
        for (int i = 0; i < 200; ++i) {
            s.x[i] = cloud.x[i] - 8.0;
            s.y[i] = cloud.y[i];
            s.z[i] = cloud.z[i];
            s.vx[i] = cloud.vx[i];
            s.vy[i] = cloud.vy[i];
            s.vz[i] = cloud.vz[i];
            s.m[i] = cloud.m[i];
        }
        const double vt = 0.5 * std::sqrt(1.0 * 2.0 / 0.08);
        s.x[200] = 7.96;
        s.x[201] = 8.04;
        s.vy[200] = -vt;
        s.vy[201] = vt;
        s.m[200] = s.m[201] = 1.0;
        const double T = 2.0, dt = 5e-3, eta = 0.02;
        auto run = [&](int scheme, long long& pevals, double& drift, double& elapsed) {  // 0 block, 1 adaptive, 2 fixed
            ngrav_gpu_ctx* ctx = MakeContext(1.0, 0.01, 0.0, 8);
            Check(ngrav_gpu_set_particles(ctx, n, s.x.data(), s.y.data(), s.z.data(), s.vx.data(), s.vy.data(),
                                          s.vz.data(), s.m.data()),
                  ctx, "set_particles");
            Check(ngrav_gpu_prime(ctx), ctx, "prime");
            const double e0 = Energy(ctx);
            Check(ngrav_gpu_reset_cumulative(ctx), ctx, "reset_cumulative");
            double t = 0.0;
            while (t < T) {
                if (scheme == 0) {
                    int rmax = 0;
                    Check(ngrav_gpu_block_step(ctx, dt, eta, 8, &rmax), ctx, "block_step");
                    t += dt;
                } else if (scheme == 1) {
                    double h = dt;
                    Check(ngrav_gpu_adaptive_dt(ctx, eta, dt, &h), ctx, "adaptive_dt");
                    Check(ngrav_gpu_step(ctx, 1, h), ctx, "step");
                    t += h;
                } else {
                    Check(ngrav_gpu_step(ctx, 1, dt), ctx, "step");
                    t += dt;
                }
            }
            pevals = StatsField(ctx, &ngrav_gpu_stats::cum_particle_evals);
            elapsed = t;
            drift = std::abs((Energy(ctx) - e0) / e0);
            ngrav_gpu_destroy(ctx);
        };
        long long pe[3];
        double dr[3], el[3];
        for (int k = 0; k < 3; ++k) run(k, pe[k], dr[k], el[k]);
        const double ratio = pe[0] > 0 ? double(pe[1]) / double(pe[0]) : 0.0;
        std::printf("  200-body cloud + 1 tight binary, integrated to t=%.1f:\n", T);
        std::printf("    fixed global    drift %.2e   %lld pevals  (t=%.2f)\n", dr[2], pe[2], el[2]);
        std::printf("    adaptive global drift %.2e   %lld pevals  (t=%.2f)\n", dr[1], pe[1], el[1]);
        std::printf("    block           drift %.2e   %lld pevals  (t=%.2f)   (%.1fx fewer than adaptive)\n", dr[0],
                    pe[0], el[0], ratio);
        CheckPrint(ok, "block-scheme energy drift", dr[0], 1e-2);
        CheckPrint(ok, "block uses >=2x fewer force evals than adaptive", ratio >= 2.0 ? 0.0 : 1.0, 0.0);
    }
    {
        ngrav_host::State s = ngrav_host::Plummer(1200, 4);
        std::fill(s.vx.begin(), s.vx.end(), 0.0);
        std::fill(s.vy.begin(), s.vy.end(), 0.0);
        std::fill(s.vz.begin(), s.vz.end(), 0.0);
        ngrav_gpu_ctx* ctx = MakeContext(1.0, 0.02, 0.5, 8);
        Check(ngrav_gpu_set_particles(ctx, (int64_t)s.Count(), s.x.data(), s.y.data(), s.z.data(), s.vx.data(),
                                      s.vy.data(), s.vz.data(), s.m.data()),
              ctx, "set_particles");
        Check(ngrav_gpu_prime(ctx), ctx, "prime");
        const double e0 = Energy(ctx);
        for (int i = 0; i < 150; ++i) {
            int rmax = 0;
            Check(ngrav_gpu_block_step(ctx, 3e-3, 0.03, 5, &rmax), ctx, "block_step");
        }
        const double drift = std::abs((Energy(ctx) - e0) / e0);
        ngrav_gpu_destroy(ctx);
        std::printf("  BH cold collapse N=1200, 150 base steps: block-scheme energy drift %.2e\n", drift);
        CheckPrint(ok, "block-scheme BH cold-collapse energy drift", drift, 0.05);
    }
    std::printf("\nrung-selftest: %s\n", ok ? "PASS" : "FAIL");
    return ok ? 0 : 1;
}

struct KeplerRun {
    double drift;
    long long evals;
};

// RunEccentric (SelfTest.cpp:391-434): an equal-mass pair on an orbit of
// eccentricity e for `periods` periods, exact pair sum, eps 1e-4; energy
// sampled every 32 steps; drift = (Emax - Emin) / |mean|.
KeplerRun RunEccentric(double e, double dt, bool adaptive, double eta, int periods) {
    const double G = 1.0, m = 1.0, r0 = 1.0;
    const double a = r0 / (1.0 + e);
    const double vRel = std::sqrt(G * 2.0 * m * (2.0 / r0 - 1.0 / a));
    const double period = 2.0 * M_PI * std::sqrt(a * a * a / (G * 2.0 * m));
    const double x[2] = {-r0 / 2, r0 / 2}, y[2] = {0, 0}, z[2] = {0, 0};
    const double vx[2] = {0, 0}, vy[2] = {-vRel / 2, vRel / 2}, vz[2] = {0, 0}, mm[2] = {m, m};
    ngrav_gpu_ctx* ctx = MakeContext(G, 1e-4, 0.0, 8);
    Check(ngrav_gpu_set_particles(ctx, 2, x, y, z, vx, vy, vz, mm), ctx, "set_particles");
    Check(ngrav_gpu_prime(ctx), ctx, "prime");
    const long long ev0 = StatsField(ctx, &ngrav_gpu_stats::force_evals);
    const double E0 = Energy(ctx);
    double Emin = E0, Emax = E0, t = 0.0;
    const double tEnd = periods * period;
    long long k = 0;
    while (t < tEnd && k < 20000000) {
        double h = dt;
        if (adaptive) Check(ngrav_gpu_adaptive_dt(ctx, eta, dt, &h), ctx, "adaptive_dt");
        Check(ngrav_gpu_step(ctx, 1, h), ctx, "step");
        t += h;
        if ((k++ % 32) == 0) {
            const double E = Energy(ctx);
            Emin = std::min(Emin, E);
            Emax = std::max(Emax, E);
        }
    }
    KeplerRun r;
    r.drift = (Emax - Emin) / std::abs(0.5 * (Emax + Emin));
    r.evals = StatsField(ctx, &ngrav_gpu_stats::force_evals) - ev0;
    ngrav_gpu_destroy(ctx);
    return r;
}

// CoreDtSelfTest (SelfTest.cpp:438-482) on the GPU path.
int DtSelfTest() {
    bool ok = true;
    std::printf("[adaptive global dt, GPU]\n");
    const KeplerRun mild = RunEccentric(0.36, 2.0 * M_PI * std::sqrt(std::pow(1.0 / 1.36, 3) / 2.0) / 2000.0, false,
                                        0.0, 4);
    CheckPrint(ok, "fixed-dt mild-orbit energy drift", mild.drift, 1e-4);
    const double aEcc = 1.0 / 1.9;
    const double Tecc = 2.0 * M_PI * std::sqrt(aEcc * aEcc * aEcc / 2.0);
    const KeplerRun ad = RunEccentric(0.9, Tecc / 600.0, true, 0.015, 3);
    std::printf("  adaptive(eta=0.015): drift=%.3e  evals=%lld\n", ad.drift, ad.evals);
    CheckPrint(ok, "adaptive e=0.9 energy drift", ad.drift, 1e-3);
    const KeplerRun c1 = RunEccentric(0.9, Tecc / 4800.0, false, 0.0, 3);
    const KeplerRun c2 = RunEccentric(0.9, Tecc / 9600.0, false, 0.0, 3);
    const double p = std::log(c1.drift / c2.drift) / std::log(2.0);
    const double div = 9600.0 * std::pow(c2.drift / ad.drift, 1.0 / p);
    const KeplerRun fm = RunEccentric(0.9, Tecc / div, false, 0.0, 3);
    std::printf("  fixed dt calibration: order p=%.2f, extrapolated div=%.0f -> verified drift=%.3e  evals=%lld\n", p,
                div, fm.drift, fm.evals);
    const double ratio = double(fm.evals) / double(std::max(1LL, ad.evals));
    std::printf("  fixed/adaptive force-eval ratio at matched accuracy = %.2f\n", ratio);
    CheckPrint(ok, "extrapolation sanity: verified drift within 50% of target", fm.drift / ad.drift - 1.0, 0.5);
    CheckPrint(ok, "adaptive uses >=2x fewer evals at matched accuracy", std::max(0.0, 2.0 - ratio), 0.0);
    std::printf("\ndt-selftest: %s\n", ok ? "PASS" : "FAIL");
    return ok ? 0 : 1;
}

void PrintValue(const fw::TomlValue& v) {
    switch (v.kind) {
        case fw::TomlValue::Table: {
            std::printf("{");
            bool first = true;
            for (const auto& [k, c] : v.table) {
                std::printf("%s\"%s\": ", first ? "" : ", ", k.c_str());
                PrintValue(*c);
                first = false;
            }
            std::printf("}");
            break;
        }
        case fw::TomlValue::Array: {
            std::printf("[");
            for (size_t i = 0; i < v.array.size(); ++i) {
                if (i) std::printf(", ");
                PrintValue(*v.array[i]);
            }
            std::printf("]");
            break;
        }
        case fw::TomlValue::String: {
            std::printf("\"");
            for (char c : v.str) {
                if (c == '"' || c == '\\') std::printf("\\%c", c);
                else if ((unsigned char)c < 0x20) std::printf("\\u%04x", (unsigned)(unsigned char)c);
                else std::printf("%c", c);
            }
            std::printf("\"");
            break;
        }
        case fw::TomlValue::Int: std::printf("%lld", (long long)v.i); break;
        case fw::TomlValue::Float:
            // JSON as Python's json module reads it (Infinity / NaN tokens).
            if (std::isnan(v.f)) std::printf("NaN");
            else if (std::isinf(v.f)) std::printf(v.f > 0 ? "Infinity" : "-Infinity");
            else {
                char buf[40];
                std::snprintf(buf, sizeof buf, "%.17g", v.f);
                std::printf("%s%s", buf, std::strpbrk(buf, ".e") ? "" : ".0");  // stays a float
            }
            break;
        case fw::TomlValue::Bool: std::printf(v.b ? "true" : "false"); break;
    }
}

}  // namespace

int main(int argc, char** argv) {
    const Args a = ParseArgs(argc, argv);
    try {
        if (!a.printDeck.empty()) {
            const fw::Deck deck = fw::Deck::FromFile(a.printDeck);
            PrintValue(deck.Root());
            std::printf("\n");
            return 0;
        }
        if (a.selftest) return SelfTest();
        if (a.rungSelftest) return RungSelfTest();
        if (a.dtSelftest) return DtSelfTest();
        if (!a.dumpIc.empty()) return a.deck.empty() ? DumpIc(a) : DumpDeckIc(a);
        if (!a.bench.empty()) return RunBench(a);
        if (a.deck.empty() || a.out.empty()) {
            std::fprintf(stderr,
                         "usage:\n"
                         "  nbody_gb300 --deck <f.toml> --out <dir> [--frames N] [--substeps N]\n"
                         "  nbody_gb300 --bench <solver> --bench-n N [--bench-theta T] [--bench-reps R]\n"
                         "  nbody_gb300 --dump-ic <file.bin> --bench-n N   (raw f32 x,y,z,m,vx,vy,vz)\n"
                         "  nbody_gb300 --selftest | --rung-selftest | --dt-selftest | --print-deck <f.toml>\n");
            return 2;
        }
        const fw::Deck deck = fw::Deck::FromFile(a.deck);
        ngrav_host::DeckSim sim;
        sim.Configure(deck);
        fw::HeadlessOptions opts;
        opts.outDir = a.out;
        opts.frames = a.frames;
        opts.substeps = a.substeps;
        return fw::RunHeadless(sim, deck, opts);
    } catch (const std::exception& e) {
        std::fprintf(stderr, "error: %s\n", e.what());
        return 1;
    }
}
