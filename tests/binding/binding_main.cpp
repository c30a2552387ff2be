// binding_main.cpp -- the reference-side binding of INTEGRATION.md, run as a
// maintainer would wire it: GpuBarnesHut (include/ngrav_gpu_accelfn.hpp)
// registered with SetAuxSolver(Solver::BarnesHut, ...) on a System whose
// ComputeAccel carries the edit INTEGRATION.md shows for the Barnes-Hut case
// (include/ngrav/System.hpp:57-66 of the reference): a registered
// Barnes-Hut evaluator is consulted first.  Test infrastructure.
//
// Usage: binding_main <n> <in.f64> <out.f64>
//   in.f64:  x, y, z, m (n doubles each) then G, eps, theta, ncrit
//   out.f64: ax, ay, az of the first evaluation, then of a second one made
//            after the registering copy of the functor has been destroyed
#include "ngrav_gpu_accelfn.hpp"

#include <cstdio>
#include <exception>
#include <unordered_map>
#include <vector>

namespace {

// The part of the reference's System<3> the binding goes through
// (System.hpp:40-78), with the edited Barnes-Hut case.
struct MiniSystem {
    std::unordered_map<int, ngrav::AccelFn<3>> m_aux;
    void SetAuxSolver(ngrav::Solver which, ngrav::AccelFn<3> fn) { m_aux[static_cast<int>(which)] = std::move(fn); }
    void ComputeAccel(ngrav::Solver solver, const ngrav::SoA<3>& in, const ngrav::StepParams& sp,
                      ngrav::SoA<3>& out) const {
        switch (solver) {
            case ngrav::Solver::BarnesHut: {
                if (auto gpu = m_aux.find(static_cast<int>(ngrav::Solver::BarnesHut)); gpu != m_aux.end()) {
                    gpu->second(in, sp, out);  // the registered GB300 path
                    return;
                }
                throw std::runtime_error("no CPU Barnes-Hut in this stand-in");
            }
            default:
                throw std::runtime_error("solver not part of the stand-in");
        }
    }
};

}  // namespace

int main(int argc, char** argv) {
    if (argc != 4) {
        std::fprintf(stderr, "usage: %s <n> <in.f64> <out.f64>\n", argv[0]);
        return 2;
    }
    try {
        const std::size_t n = std::stoul(argv[1]);
        std::vector<double> buf(4 * n + 4);
        FILE* f = std::fopen(argv[2], "rb");
        if (!f || std::fread(buf.data(), sizeof(double), buf.size(), f) != buf.size()) return 3;
        std::fclose(f);
        ngrav::SoA<3> s;
        s.x.assign(buf.begin(), buf.begin() + n);
        s.y.assign(buf.begin() + n, buf.begin() + 2 * n);
        s.z.assign(buf.begin() + 2 * n, buf.begin() + 3 * n);
        s.m.assign(buf.begin() + 3 * n, buf.begin() + 4 * n);
        ngrav::StepParams sp;
        sp.G = buf[4 * n];
        sp.soft = ngrav::Softening::Plummer(buf[4 * n + 1]);
        sp.mac.theta = buf[4 * n + 2];
        const int ncrit = (int)buf[4 * n + 3];

        MiniSystem sys;
        {
            ngrav_gpu::GpuBarnesHut gpu(sp, ncrit);
            sys.SetAuxSolver(ngrav::Solver::BarnesHut, gpu);  // stores a copy
        }  // the original is gone; the copy inside the std::function keeps the context
        std::vector<double> out;
        for (int pass = 0; pass < 2; ++pass) {
            ngrav::SoA<3> acc;
            sys.ComputeAccel(ngrav::Solver::BarnesHut, s, sp, acc);
            out.insert(out.end(), acc.ax.begin(), acc.ax.end());
            out.insert(out.end(), acc.ay.begin(), acc.ay.end());
            out.insert(out.end(), acc.az.begin(), acc.az.end());
        }
        f = std::fopen(argv[3], "wb");
        if (!f || std::fwrite(out.data(), sizeof(double), out.size(), f) != out.size()) return 4;
        std::fclose(f);
    } catch (const std::exception& e) {
        std::fprintf(stderr, "binding_main: %s\n", e.what());
        return 1;
    }
    return 0;
}
