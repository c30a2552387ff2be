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

// The Barnes-Hut gates of the reference self-test (SelfTest.cpp:43-74 and
// :212-265) on the GPU path, with FP32 tolerances: theta = 0 equals the
// exact sum; the quadrupole cuts the max error at theta = 0.5 >= 3x.
int SelfTest() {
    bool ok = true;
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
