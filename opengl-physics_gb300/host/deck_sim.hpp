// deck_sim.hpp -- the N-body fw::Simulation over the GPU C-ABI.
//
// Drop-in for ngrav::DeckSim<3> (projects/nbody_core/include/ngrav/
// DeckSim.hpp:23-68, src/DeckSim.cpp): the same deck keys, the same
// scenario / deck-override rule, the same frame fields ("pos", "vel" as
// N x 3 float32) and the same diagnostics columns, with the force/step path
// on the GPU through include/ngrav_gpu.h instead of System<3>.
#pragma once

#include "deck.hpp"
#include "ngrav_gpu.h"
#include "scenarios.hpp"
#include "simulation.hpp"

#include <string>
#include <vector>

namespace ngrav_host {

class DeckSim : public fw::Simulation {
public:
    DeckSim() = default;
    ~DeckSim() override;
    DeckSim(const DeckSim&) = delete;
    DeckSim& operator=(const DeckSim&) = delete;

    void Configure(const fw::Deck& deck) override;
    void Reset() override;
    void Step(int substeps) override;
    void Snapshot(fw::OutputWriter& writer) override;
    fw::SimInfo Info() const override;

    ngrav_gpu_ctx* Context() const { return m_ctx; }
    const std::vector<std::string>& Warnings() const { return m_warnings; }

private:
    void LoadScenario();
    void Check(int rc, const char* what) const;

    ngrav_gpu_ctx* m_ctx = nullptr;
    ngrav_gpu_opts m_opts{};
    std::string m_title = "N-Body Gravity";
    std::string m_scenarioType = "plummer";
    ScenarioParams m_params;
    int m_substepsPerFrame = 4;
    double m_dt = 1e-3;
    double m_time = 0.0;
    long m_step = 0;
    double m_lastDt = 0.0;
    double m_energy0 = 0.0;
    double m_lmag0 = 0.0;
    bool m_deckHasG = false, m_deckHasEps = false, m_deckHasDt = false;
    double m_deckG = 1.0, m_deckEps = 0.05, m_deckDt = 1e-3;
    long long m_n = 0;
    bool m_adaptive = false, m_block = false, m_spline = false;
    double m_eta = 0.03, m_alpha = 0.001;
    int m_blockMaxRung = 8;
    int m_rungMax = 0;
    std::vector<std::string> m_warnings;
    std::vector<float> m_pos, m_vel;  // frame buffers, reused across snapshots
};

}  // namespace ngrav_host
