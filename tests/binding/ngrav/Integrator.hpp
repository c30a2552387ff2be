// Stand-in for the reference's ngrav/Integrator.hpp and the headers it pulls
// in (State.hpp, Solvers.hpp, Mac.hpp, Softening.hpp): only the declarations
// the AccelFn adapter (include/ngrav_gpu_accelfn.hpp) and the edited
// System<3>::ComputeAccel touch, with the reference's names, members and
// defaults (State.hpp:16-46, Solvers.hpp:11-40, Mac.hpp:13-22,
// Softening.hpp:30-33,120-140, Integrator.hpp:13-14).  Lets the tests compile
// the adapter exactly as a maintainer would, without the reference's tree.
#pragma once

#include <cstddef>
#include <functional>
#include <vector>

namespace ngrav {

enum class SofteningKind { Plummer, Spline };
struct Softening {
    SofteningKind kind = SofteningKind::Plummer;
    double eps = 0.05;
    double eps2 = 0.05 * 0.05;
    static Softening Plummer(double e) { return Softening{SofteningKind::Plummer, e, e * e}; }
    static Softening Spline(double h) { return Softening{SofteningKind::Spline, h, h * h}; }
};

enum class MacKind { Geometric, Relative };
struct MacParams {
    MacKind kind = MacKind::Geometric;
    double theta = 0.5;
    double alpha = 0.001;
};

enum class Solver { Direct, BarnesHut, Fmm, SphericalFmm, ComplexFmm };

struct StepParams {
    double G = 1.0;
    Softening soft = Softening::Plummer(0.05);
    double dt = 1e-3;
    MacParams mac{};
    Solver solver = Solver::BarnesHut;
};

template <int D>
struct SoA {
    std::vector<double> x, y, z, vx, vy, vz, m, ax, ay, az;
    std::size_t Count() const { return x.size(); }
    void ResizeAccel(std::size_t n) {
        ax.assign(n, 0.0);
        ay.assign(n, 0.0);
        if constexpr (D == 3) az.assign(n, 0.0);
    }
};

template <int D>
using AccelFn = std::function<void(const SoA<D>& in, const StepParams& sp, SoA<D>& out)>;

}  // namespace ngrav
