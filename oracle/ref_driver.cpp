// C-ABI driver around the reference's own CPU implementation of the
// Barnes-Hut path (projects/nbody_core), compiled from the reference sources
// in place by oracle/build_ref.sh into oracle/_ref/libngrav_ref.so.
//
// TEST INFRASTRUCTURE ONLY. This file is the checker's window onto the real
// reference: tests/golden/make_golden.py calls it to produce the golden
// fixtures that pin the C restatement (oracle/ngrav_oracle.c) and the CUDA
// path. The product library never links or loads it.
//
// Every entry point forwards to the reference's public API unchanged:
//   ref_plummer         -> ngrav::ic::Plummer<3>            (include/ngrav/ic/Plummer.hpp:26-112)
//   ref_direct_accel    -> ngrav::ComputeAccelDirect<3>      (src/Solvers.cpp:77-106)
//   ref_bh_accel        -> AdaptiveTree<3>(v, ncrit) + ComputeQuadrupoles + ComputeAccelBarnesHut<3>
//                          (src/Tree.cpp:33-52,205-254; src/Solvers.cpp:407-415)
//   ref_bh_pp_accel     -> the per-particle walk: relative MAC (src/Solvers.cpp:359-382) or
//                          geometric on a target subset (:384-405)
//   ref_tree_*          -> AdaptiveTree<3> node arrays      (include/ngrav/Tree.hpp:44-63)
//   ref_leapfrog        -> ngrav::LeapfrogStep<3>           (src/Integrator.cpp:9-39)
//   ref_scenario        -> ngrav::BuildScenario<3>(ScenarioFromString(type), params)
//                          (src/Scenarios.cpp:355-384)
//   ref_diagnostics     -> System<3>::TotalEnergy / CenterOfMass / AngularMomentum
//                          (include/ngrav/System.hpp:119-193) and the momentum sum of
//                          DeckSim::Snapshot (src/DeckSim.cpp:147-153)
#include "ngrav/Integrator.hpp"
#include "ngrav/Scenarios.hpp"
#include "ngrav/Solvers.hpp"
#include "ngrav/System.hpp"
#include "ngrav/Tree.hpp"
#include "ngrav/ic/Plummer.hpp"

#include <algorithm>
#include <chrono>
#include <cmath>
#include <cstdint>
#include <cstring>
#include <random>
#include <vector>

using namespace ngrav;

namespace {

SoA<3> MakeSoA(int n, const double* x, const double* y, const double* z, const double* m) {
    SoA<3> s;
    s.Resize(static_cast<std::size_t>(n));
    for (int i = 0; i < n; ++i) {
        s.x[i] = x[i];
        s.y[i] = y[i];
        s.z[i] = z[i];
        s.m[i] = m[i];
    }
    return s;
}

int g_soft_kind = 0;  // 0 Plummer, 1 spline (ref_set_softening)

StepParams MakeParams(double G, double eps, double theta) {
    StepParams sp;
    sp.G = G;
    sp.soft = g_soft_kind == 1 ? Softening::Spline(eps) : Softening::Plummer(eps);
    sp.mac.theta = theta;
    sp.mac.kind = MacKind::Geometric;
    sp.solver = Solver::BarnesHut;
    return sp;
}

struct TreeHandle {
    AdaptiveTree<3>* tree;
};

} // namespace

extern "C" {

// Softening kind of every later call: 0 Plummer, 1 spline (Softening.hpp:125-139).
void ref_set_softening(int kind) { g_soft_kind = kind; }


int ref_plummer(int n, unsigned seed, double* x, double* y, double* z, double* vx, double* vy, double* vz,
                double* m) {
    ic::PlummerParams pp;
    pp.n = n;
    pp.seed = seed;
    const SoA<3> s = ic::Plummer<3>(pp);
    for (int i = 0; i < n; ++i) {
        x[i] = s.x[i];
        y[i] = s.y[i];
        z[i] = s.z[i];
        vx[i] = s.vx[i];
        vy[i] = s.vy[i];
        vz[i] = s.vz[i];
        m[i] = s.m[i];
    }
    return 0;
}

// Input cloud of the reference's BH-vs-Direct self-test (src/SelfTest.cpp:43-57):
// uniform in [-1,1]^3, m = 0.5 + 0.5 (u + 1), std::mt19937(seed).
void ref_cloud_uniform(int n, unsigned seed, double* x, double* y, double* z, double* m) {
    std::mt19937 rng(seed);
    std::uniform_real_distribution<double> u(-1.0, 1.0);
    for (int i = 0; i < n; ++i) {
        x[i] = u(rng);
        y[i] = u(rng);
        z[i] = u(rng);
        m[i] = 0.5 + 0.5 * (u(rng) + 1.0);
    }
}

// Input cloud of the reference's quadrupole self-test (src/SelfTest.cpp:212-227):
// uniform in the unit ball (r = cbrt(u)), m = 1/n, std::mt19937(seed).
void ref_cloud_ball(int n, unsigned seed, double* x, double* y, double* z, double* m) {
    std::mt19937 rng(seed);
    std::uniform_real_distribution<double> uni(0.0, 1.0);
    for (int i = 0; i < n; ++i) {
        const double r = std::cbrt(uni(rng));
        const double cosT = 2.0 * uni(rng) - 1.0, sinT = std::sqrt(std::max(0.0, 1.0 - cosT * cosT));
        const double phi = 2.0 * M_PI * uni(rng);
        x[i] = r * sinT * std::cos(phi);
        y[i] = r * sinT * std::sin(phi);
        z[i] = r * cosT;
        m[i] = 1.0 / n;
    }
}

void ref_direct_accel(int n, const double* x, const double* y, const double* z, const double* m, double G,
                      double eps, double* ax, double* ay, double* az) {
    const SoA<3> s = MakeSoA(n, x, y, z, m);
    SoA<3> out;
    ComputeAccelDirect<3>(ViewOf(s), MakeParams(G, eps, 0.5), out);
    std::memcpy(ax, out.ax.data(), sizeof(double) * n);
    std::memcpy(ay, out.ay.data(), sizeof(double) * n);
    std::memcpy(az, out.az.data(), sizeof(double) * n);
}

// quad != 0: monopole + quadrupole (the deck/System path); quad == 0: monopole only.
// Returns the wall time of the tree build + quadrupoles + walk in milliseconds.
double ref_bh_accel(int n, const double* x, const double* y, const double* z, const double* m, double G, double eps,
                    double theta, int ncrit, int quad, double* ax, double* ay, double* az) {
    const SoA<3> s = MakeSoA(n, x, y, z, m);
    const PosMassView<3> v = ViewOf(s);
    const StepParams sp = MakeParams(G, eps, theta);
    SoA<3> out;
    const auto t0 = std::chrono::steady_clock::now();
    AdaptiveTree<3> tree(v, ncrit);
    if (quad) tree.ComputeQuadrupoles(v);
    ComputeAccelBarnesHut<3>(v, sp, tree, {}, out);
    const auto t1 = std::chrono::steady_clock::now();
    std::memcpy(ax, out.ax.data(), sizeof(double) * n);
    std::memcpy(ay, out.ay.data(), sizeof(double) * n);
    std::memcpy(az, out.az.data(), sizeof(double) * n);
    return std::chrono::duration<double, std::milli>(t1 - t0).count();
}

// The relative-MAC walk: ComputeAccelBarnesHut with MacKind::Relative and the
// previous |a| per particle (Solvers.cpp:407-415 -> :359-382), or, with
// targets != NULL, the geometric per-particle walk on the particles whose
// flag is set (ComputeAccelBarnesHutTargets, :384-405).
void ref_bh_pp_accel(int n, const double* x, const double* y, const double* z, const double* m, double G,
                     double eps, double theta, int ncrit, double alpha, const double* aold,
                     const unsigned char* targets, double* ax, double* ay, double* az) {
    const SoA<3> s = MakeSoA(n, x, y, z, m);
    const PosMassView<3> v = ViewOf(s);
    StepParams sp = MakeParams(G, eps, theta);
    sp.mac.kind = MacKind::Relative;
    sp.mac.alpha = alpha;
    AdaptiveTree<3> tree(v, ncrit);
    tree.ComputeQuadrupoles(v);
    SoA<3> out;
    out.ResizeAccel(static_cast<std::size_t>(n));
    if (targets) {
        std::vector<int> tg;
        for (int i = 0; i < n; ++i)
            if (targets[i]) tg.push_back(i);
        ComputeAccelBarnesHutTargets<3>(v, MakeParams(G, eps, theta), tree, tg, out);
    } else {
        std::vector<double> a(aold, aold + n);
        ComputeAccelBarnesHut<3>(v, sp, tree, a, out);
    }
    std::memcpy(ax, out.ax.data(), sizeof(double) * n);
    std::memcpy(ay, out.ay.data(), sizeof(double) * n);
    std::memcpy(az, out.az.data(), sizeof(double) * n);
}

void* ref_tree_build(int n, const double* x, const double* y, const double* z, const double* m, int ncrit,
                     int maxDepth, int* numNodes) {
    const SoA<3> s = MakeSoA(n, x, y, z, m);
    const PosMassView<3> v = ViewOf(s);
    auto* h = new TreeHandle{new AdaptiveTree<3>(v, ncrit, maxDepth)};
    h->tree->ComputeQuadrupoles(v);
    *numNodes = h->tree->NumNodes();
    return h;
}

// Node arrays in the reference's own (creation-order) numbering plus the
// derived (level, octant-path prefix, subtree count) needed for a canonical,
// numbering-independent comparison. prefix holds 3 bits per level, root = 0.
void ref_tree_export(void* handle, int n, int* level, unsigned long long* prefix, int* count, int* isLeaf,
                     double* center, double* half, double* com, double* mass, double* maxRadius, double* quad,
                     int* order, int* parent, int* firstParticle) {
    const AdaptiveTree<3>& t = *static_cast<TreeHandle*>(handle)->tree;
    const int nn = t.NumNodes();
    std::vector<int> cnt(static_cast<std::size_t>(nn), 0);
    for (int i = 0; i < nn; ++i) {
        if (t.IsLeaf(i)) cnt[i] = t.particleCount[i];
    }
    for (int i = nn - 1; i > 0; --i) cnt[t.parent[i]] += cnt[i];
    for (int i = 0; i < nn; ++i) {
        if (i == 0) {
            level[i] = 0;
            prefix[i] = 0ull;
        } else {
            const int p = t.parent[i];
            int oct = -1;
            for (int c = 0; c < 8; ++c)
                if (t.children[p][c] == i) oct = c;
            level[i] = level[p] + 1;
            prefix[i] = (prefix[p] << 3) | static_cast<unsigned long long>(oct);
        }
        count[i] = cnt[i];
        isLeaf[i] = t.IsLeaf(i) ? 1 : 0;
        center[3 * i + 0] = t.center[i].x;
        center[3 * i + 1] = t.center[i].y;
        center[3 * i + 2] = t.center[i].z;
        half[i] = t.halfSize[i];
        com[3 * i + 0] = t.com[i].x;
        com[3 * i + 1] = t.com[i].y;
        com[3 * i + 2] = t.com[i].z;
        mass[i] = t.mass[i];
        maxRadius[i] = t.maxRadius[i];
        quad[5 * i + 0] = t.Qxx[i];
        quad[5 * i + 1] = t.Qyy[i];
        quad[5 * i + 2] = t.Qxy[i];
        quad[5 * i + 3] = t.Qxz[i];
        quad[5 * i + 4] = t.Qyz[i];
        parent[i] = t.parent[i];
        firstParticle[i] = t.firstParticle[i];
    }
    for (int k = 0; k < n; ++k) order[k] = t.order[k];
}

void ref_tree_free(void* handle) {
    auto* h = static_cast<TreeHandle*>(handle);
    delete h->tree;
    delete h;
}

// KDK leapfrog through the reference's LeapfrogStep with a Barnes-Hut
// AccelFn at leaf capacity `ncrit` (the System path hard-wires ncrit 8,
// include/ngrav/System.hpp:57). If primed == 0 the acceleration is computed
// first, as System::Prime does. State arrays are updated in place. Returns
// the wall time of the nsteps steps in milliseconds.
double ref_leapfrog(int n, double* x, double* y, double* z, double* vx, double* vy, double* vz, const double* m,
                    double* ax, double* ay, double* az, double G, double eps, double theta, int ncrit, double dt,
                    int nsteps, int primed) {
    SoA<3> s = MakeSoA(n, x, y, z, m);
    for (int i = 0; i < n; ++i) {
        s.vx[i] = vx[i];
        s.vy[i] = vy[i];
        s.vz[i] = vz[i];
        s.ax[i] = ax[i];
        s.ay[i] = ay[i];
        s.az[i] = az[i];
    }
    StepParams sp = MakeParams(G, eps, theta);
    sp.dt = dt;
    const AccelFn<3> accel = [ncrit](const SoA<3>& in, const StepParams& p, SoA<3>& o) {
        const PosMassView<3> v = ViewOf(in);
        AdaptiveTree<3> tree(v, ncrit);
        tree.ComputeQuadrupoles(v);
        ComputeAccelBarnesHut<3>(v, p, tree, {}, o);
    };
    if (!primed) {
        SoA<3> tmp;
        accel(s, sp, tmp);
        s.ax = tmp.ax;
        s.ay = tmp.ay;
        s.az = tmp.az;
    }
    SoA<3> scratch;
    const auto t0 = std::chrono::steady_clock::now();
    for (int k = 0; k < nsteps; ++k) LeapfrogStep<3>(s, sp, accel, scratch);
    const auto t1 = std::chrono::steady_clock::now();
    for (int i = 0; i < n; ++i) {
        x[i] = s.x[i];
        y[i] = s.y[i];
        z[i] = s.z[i];
        vx[i] = s.vx[i];
        vy[i] = s.vy[i];
        vz[i] = s.vz[i];
        ax[i] = s.ax[i];
        ay[i] = s.ay[i];
        az[i] = s.az[i];
    }
    return std::chrono::duration<double, std::milli>(t1 - t0).count();
}

// nsteps block (power-of-two rung) steps through System::Step with
// StepParams::block (include/ngrav/System.hpp:89-98 -> BlockStep :239-294),
// Barnes-Hut, primed by System::Prime from the positions.  The state and a
// are updated in place; rung[i] receives the rungs of the last step.
void ref_block_step(int n, double* x, double* y, double* z, double* vx, double* vy, double* vz, const double* m,
                    double* ax, double* ay, double* az, double G, double eps, double theta, double dt, double eta,
                    int max_rung, int nsteps, int* rung) {
    SoA<3> s = MakeSoA(n, x, y, z, m);
    for (int i = 0; i < n; ++i) {
        s.vx[i] = vx[i];
        s.vy[i] = vy[i];
        s.vz[i] = vz[i];
    }
    System<3> sys;
    sys.SetParticles(std::move(s));
    StepParams sp = MakeParams(G, eps, theta);
    sp.dt = dt;
    sp.block = true;
    sp.eta = eta;
    sp.blockMaxRung = max_rung;
    sys.Prime(sp);
    for (int k = 0; k < nsteps; ++k) sys.Step(sp);
    const SoA<3>& st = sys.State();
    for (int i = 0; i < n; ++i) {
        x[i] = st.x[i];
        y[i] = st.y[i];
        z[i] = st.z[i];
        vx[i] = st.vx[i];
        vy[i] = st.vy[i];
        vz[i] = st.vz[i];
        ax[i] = st.ax[i];
        ay[i] = st.ay[i];
        az[i] = st.az[i];
    }
    const std::span<const int> r = sys.Rungs();
    for (int i = 0; i < n; ++i) rung[i] = i < static_cast<int>(r.size()) ? r[i] : 0;
}

// out[0] = total energy (O(N^2) potential), out[1..3] = centre of mass,
// out[4..6] = angular momentum about the COM, out[7..9] = linear momentum.
void ref_diagnostics(int n, const double* x, const double* y, const double* z, const double* vx, const double* vy,
                     const double* vz, const double* m, double G, double eps, double* out) {
    SoA<3> s = MakeSoA(n, x, y, z, m);
    for (int i = 0; i < n; ++i) {
        s.vx[i] = vx[i];
        s.vy[i] = vy[i];
        s.vz[i] = vz[i];
    }
    System<3> sys;
    sys.SetParticles(std::move(s));
    const StepParams sp = MakeParams(G, eps, 0.5);
    out[0] = sys.TotalEnergy(sp);
    const glm::dvec3 c = sys.CenterOfMass();
    out[1] = c.x;
    out[2] = c.y;
    out[3] = c.z;
    const glm::dvec3 L = sys.AngularMomentum();
    out[4] = L.x;
    out[5] = L.y;
    out[6] = L.z;
    const SoA<3>& st = sys.State();
    double px = 0.0, py = 0.0, pz = 0.0;
    for (int i = 0; i < n; ++i) {
        px += st.m[i] * st.vx[i];
        py += st.m[i] * st.vy[i];
        pz += st.m[i] * st.vz[i];
    }
    out[7] = px;
    out[8] = py;
    out[9] = pz;
}

// The deck scenario generator.  Call with cap = 0 to learn the particle count
// (returned); then with cap >= count to receive the arrays.  params[0..2] =
// G, softening eps, suggested dt.  Returns -1 on an exception.
int ref_scenario(const char* type, int n, unsigned seed, const char* ic_file, int cap, double* x, double* y,
                 double* z, double* vx, double* vy, double* vz, double* m, double* params) {
    try {
        ScenarioParams pp;
        pp.n = n;
        pp.seed = seed;
        pp.icFile = ic_file ? ic_file : "";
        const Scenario<3> sc = BuildScenario<3>(ScenarioFromString(type, ScenarioType::PlummerSphere), pp);
        const int count = static_cast<int>(sc.state.x.size());
        if (cap >= count) {
            for (int i = 0; i < count; ++i) {
                x[i] = sc.state.x[i];
                y[i] = sc.state.y[i];
                z[i] = sc.state.z[i];
                vx[i] = sc.state.vx[i];
                vy[i] = sc.state.vy[i];
                vz[i] = sc.state.vz[i];
                m[i] = sc.state.m[i];
            }
        }
        params[0] = sc.G;
        params[1] = sc.soft.eps;
        params[2] = sc.suggestedDt;
        return count;
    } catch (...) {
        return -1;
    }
}

} // extern "C"
