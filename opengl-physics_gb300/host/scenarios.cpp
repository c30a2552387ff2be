// scenarios.cpp -- see scenarios.hpp.
#include "scenarios.hpp"

#include <algorithm>
#include <cmath>
#include <fstream>
#include <random>
#include <stdexcept>

namespace ngrav_host {

namespace {
constexpr double kPi = 3.14159265358979323846;
}

State Plummer(int n, uint32_t seed, double totalMass, double scaleRadius, double G) {
    State s;
    s.Resize((size_t)n);
    std::mt19937 rng(seed);
    std::uniform_real_distribution<double> u(0.0, 1.0);
    const double m = totalMass / n;
    const double vUnit = std::sqrt(G * totalMass / scaleRadius);
    for (int i = 0; i < n; ++i) {
        const double x1 = u(rng);
        double r = 1.0 / std::sqrt(std::pow(x1, -2.0 / 3.0) - 1.0);
        r = std::min(r, 20.0);  // the reference clips the far tail
        const double cosT = 2.0 * u(rng) - 1.0;
        const double sinT = std::sqrt(std::max(0.0, 1.0 - cosT * cosT));
        const double phi = 2.0 * kPi * u(rng);
        const double rs = r * scaleRadius;
        s.x[i] = sinT * std::cos(phi) * rs;
        s.y[i] = sinT * std::sin(phi) * rs;
        s.z[i] = cosT * rs;
        double q, g;
        do {  // von Neumann rejection on g(q) = q^2 (1 - q^2)^3.5, envelope 0.1
            q = u(rng);
            g = u(rng) * 0.1;
        } while (g > q * q * std::pow(1.0 - q * q, 3.5));
        const double vEsc = std::sqrt(2.0) * std::pow(1.0 + r * r, -0.25);
        const double speed = q * vEsc;
        const double vc = 2.0 * u(rng) - 1.0;
        const double vs = std::sqrt(std::max(0.0, 1.0 - vc * vc));
        const double vphi = 2.0 * kPi * u(rng);
        const double vsp = speed * vUnit;
        s.vx[i] = vs * std::cos(vphi) * vsp;
        s.vy[i] = vs * std::sin(vphi) * vsp;
        s.vz[i] = vc * vsp;
        s.m[i] = m;
    }
    // recentre to zero COM position and momentum
    double cp[3] = {0, 0, 0}, cv[3] = {0, 0, 0}, tm = 0.0;
    for (int i = 0; i < n; ++i) {
        cp[0] += s.m[i] * s.x[i];
        cp[1] += s.m[i] * s.y[i];
        cp[2] += s.m[i] * s.z[i];
        cv[0] += s.m[i] * s.vx[i];
        cv[1] += s.m[i] * s.vy[i];
        cv[2] += s.m[i] * s.vz[i];
        tm += s.m[i];
    }
    for (double& c : cp) c /= tm;
    for (double& c : cv) c /= tm;
    for (int i = 0; i < n; ++i) {
        s.x[i] -= cp[0];
        s.y[i] -= cp[1];
        s.z[i] -= cp[2];
        s.vx[i] -= cv[0];
        s.vy[i] -= cv[1];
        s.vz[i] -= cv[2];
    }
    return s;
}

namespace {

// Cluster (Scenarios.cpp:103-143): uniform ball radius R = 1, Gaussian
// velocities of 0.3 sqrt(GM/R).
State ClusterState(int n, uint32_t seed) {
    State s;
    s.Resize((size_t)n);
    std::mt19937 rng(seed);
    std::uniform_real_distribution<double> u(0.0, 1.0);
    std::normal_distribution<double> gauss(0.0, 1.0);
    const double R = 1.0, M = 1.0, G = 1.0;
    for (int i = 0; i < n; ++i) {
        const double radius = R * std::cbrt(u(rng));
        const double cosT = 2.0 * u(rng) - 1.0, sinT = std::sqrt(std::max(0.0, 1.0 - cosT * cosT));
        const double phi = 2.0 * kPi * u(rng);
        s.x[i] = sinT * std::cos(phi) * radius;
        s.y[i] = sinT * std::sin(phi) * radius;
        s.z[i] = cosT * radius;
        const double vScale = std::sqrt(G * M / R);
        s.vx[i] = 0.3 * vScale * gauss(rng);
        s.vy[i] = 0.3 * vScale * gauss(rng);
        s.vz[i] = 0.3 * vScale * gauss(rng);
        s.m[i] = M / n;
    }
    return s;
}

}  // namespace

Scenario BuildScenario(const std::string& type, const ScenarioParams& p, bool* fellBack) {
    Scenario sc;
    const int n = std::max(p.n, 1);
    if (fellBack) *fellBack = false;
    if (type == "cluster" || type == "cold_collapse") {
        sc.state = ClusterState(n, p.seed);
        const double meanSpacing = 1.0 / std::cbrt((double)n);
        if (type == "cluster") {
            sc.name = "Cluster (N stress test)";
            sc.eps = 2.0 * meanSpacing;
            sc.suggestedDt = 1.0 / 1000.0;
        } else {  // ColdUniform (Scenarios.cpp:201-215): cluster positions at rest
            sc.name = "Cold collapse";
            std::fill(sc.state.vx.begin(), sc.state.vx.end(), 0.0);
            std::fill(sc.state.vy.begin(), sc.state.vy.end(), 0.0);
            std::fill(sc.state.vz.begin(), sc.state.vz.end(), 0.0);
            sc.eps = std::max(0.01, 1.0 * meanSpacing);
            sc.suggestedDt = 1.0 / 2000.0;
        }
        return sc;
    }
    if (type == "ic_file") {  // Scenarios.cpp:292-329
        sc.name = "IC file (raw float32 dump)";
        sc.state = ReadIcFile(p.icFile);
        sc.eps = 0.05;
        sc.suggestedDt = 1e-3;
        return sc;
    }
    if (!(type == "plummer" || type == "plummer_sphere") && fellBack) *fellBack = true;
    // PlummerEquilibrium (Scenarios.cpp:184-198)
    sc.name = "Plummer sphere (equilibrium)";
    sc.state = Plummer(n, p.seed);
    sc.eps = std::max(0.01, 1.5 * (1.0 / std::cbrt((double)n)));
    sc.suggestedDt = (2.0 * kPi) / 800.0;
    return sc;
}

State ReadIcFile(const std::string& path) {
    std::ifstream f(path, std::ios::binary | std::ios::ate);
    if (!f) throw std::runtime_error("ic_file: cannot open '" + path + "'");
    const std::streamsize bytes = f.tellg();
    f.seekg(0);
    const int n = (int)(bytes / (7 * (std::streamsize)sizeof(float)));
    if (n <= 0) throw std::runtime_error("ic_file: '" + path + "' has no particles");
    std::vector<float> raw((size_t)n * 7);
    f.read(reinterpret_cast<char*>(raw.data()), (std::streamsize)(raw.size() * sizeof(float)));
    State s;
    s.Resize((size_t)n);
    for (int i = 0; i < n; ++i) {
        const float* r = &raw[(size_t)i * 7];
        s.x[i] = r[0];
        s.y[i] = r[1];
        s.z[i] = r[2];
        s.m[i] = r[3];
        s.vx[i] = r[4];
        s.vy[i] = r[5];
        s.vz[i] = r[6];
    }
    return s;
}

void WriteIcFile(const std::string& path, const State& s) {
    std::ofstream f(path, std::ios::binary);
    if (!f) throw std::runtime_error("dump-ic: cannot open '" + path + "' for writing");
    for (size_t i = 0; i < s.Count(); ++i) {
        const float r[7] = {(float)s.x[i], (float)s.y[i], (float)s.z[i], (float)s.m[i],
                            (float)s.vx[i], (float)s.vy[i], (float)s.vz[i]};
        f.write(reinterpret_cast<const char*>(r), sizeof(r));
    }
}

State UniformCubeCloud(int n, uint32_t seed) {
    State s;
    s.Resize((size_t)n);
    std::mt19937 rng(seed);
    std::uniform_real_distribution<double> u(-1.0, 1.0);
    for (int i = 0; i < n; ++i) {
        s.x[i] = u(rng);
        s.y[i] = u(rng);
        s.z[i] = u(rng);
        s.m[i] = 0.5 + 0.5 * (u(rng) + 1.0);
    }
    return s;
}

State UniformBallCloud(int n, uint32_t seed) {
    State s;
    s.Resize((size_t)n);
    std::mt19937 rng(seed);
    std::uniform_real_distribution<double> uni(0.0, 1.0);
    for (int i = 0; i < n; ++i) {
        const double r = std::cbrt(uni(rng));
        const double cosT = 2.0 * uni(rng) - 1.0, sinT = std::sqrt(std::max(0.0, 1.0 - cosT * cosT));
        const double phi = 2.0 * kPi * uni(rng);
        s.x[i] = r * sinT * std::cos(phi);
        s.y[i] = r * sinT * std::sin(phi);
        s.z[i] = r * cosT;
        s.m[i] = 1.0 / n;
    }
    return s;
}

}  // namespace ngrav_host
