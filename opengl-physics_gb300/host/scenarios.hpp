// scenarios.hpp -- initial conditions for deck-driven runs.
//
// Restates the reference's scenario generators for the deck path
// (projects/nbody_core/src/Scenarios.cpp, include/ngrav/ic/Plummer.hpp) with
// the same std::mt19937 + <random> draw order, so a deck produces the same
// particles it does in the reference (same standard library).  Scenario names
// follow ScenarioFromString (Scenarios.cpp:358-370); unsupported ones fall
// back to the Plummer sphere, as the reference falls back on unknown names.
#pragma once

#include <cstdint>
#include <string>
#include <vector>

namespace ngrav_host {

struct State {
    std::vector<double> x, y, z, vx, vy, vz, m;
    size_t Count() const { return x.size(); }
    void Resize(size_t n) {
        for (auto* v : {&x, &y, &z, &vx, &vy, &vz, &m}) v->assign(n, 0.0);
    }
};

struct ScenarioParams {
    int n = 2000;
    uint32_t seed = 1;
    std::string icFile;
};

struct Scenario {
    State state;
    double G = 1.0;
    double eps = 0.05;          // Plummer softening length
    double suggestedDt = 1e-3;
    double suggestedTheta = 0.5;
    std::string name;
};

// type: "plummer" | "plummer_sphere" | "cluster" | "cold_collapse" | "ic_file";
// anything else -> Plummer (with `fellBack` set).
Scenario BuildScenario(const std::string& type, const ScenarioParams& p, bool* fellBack = nullptr);

// Plummer sphere in G = M = a = 1 units (ic/Plummer.hpp:26-112).
State Plummer(int n, uint32_t seed, double totalMass = 1.0, double scaleRadius = 1.0, double G = 1.0);

// The raw float32 interchange format: n records of x, y, z, m, vx, vy, vz
// (Scenarios.cpp:292-329 reader, main.cpp:253-280 writer).
State ReadIcFile(const std::string& path);
void WriteIcFile(const std::string& path, const State& s);

// Input clouds of the reference self-tests (SelfTest.cpp:43-57 and :212-227).
State UniformCubeCloud(int n, uint32_t seed);   // [-1,1]^3, m = 0.5 + 0.5 (u + 1)
State UniformBallCloud(int n, uint32_t seed);   // unit ball, m = 1/n

}  // namespace ngrav_host
