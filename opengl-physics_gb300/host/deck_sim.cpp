// deck_sim.cpp -- see deck_sim.hpp.  Deck keys follow src/DeckSim.cpp:25-74;
// GPU-only knobs are new keys: solver.leaf_capacity (ncrit, default 8 as in
// Tree.hpp:38), solver.quadrupole (default true) and precision.mode
// ("split" | "plain").
#include "deck_sim.hpp"

#include <algorithm>
#include <cmath>
#include <cstdio>
#include <stdexcept>

namespace ngrav_host {

DeckSim::~DeckSim() {
    if (m_ctx) ngrav_gpu_destroy(m_ctx);
}

void DeckSim::Check(int rc, const char* what) const {
    if (rc != NGRAV_OK) {
        const char* msg = m_ctx ? ngrav_gpu_last_error(m_ctx) : "";
        throw std::runtime_error(std::string(what) + " failed (" + std::to_string(rc) + "): " + msg);
    }
}

void DeckSim::Configure(const fw::Deck& deck) {
    m_warnings.clear();
    m_title = deck.GetString("title", "N-Body Gravity");
    auto warn = [&](const std::string& w) {
        m_warnings.push_back(w);
        std::fprintf(stderr, "warning: %s\n", w.c_str());
    };
    // time.adaptive / time.eta / time.scheme / time.block_max_rung
    // (DeckSim.cpp:27-35); block timesteps need a solver with a target-subset
    // form (Direct / Barnes-Hut, System.hpp:93-98), else the adaptive or
    // global scheme runs.
    m_adaptive = deck.GetBool("time.adaptive", false);
    m_eta = deck.GetDouble("time.eta", 0.03);
    m_blockMaxRung = std::max(0, deck.GetInt("time.block_max_rung", 8));
    m_substepsPerFrame = deck.GetInt("time.substeps_per_frame", 4);

    ngrav_gpu_default_opts(&m_opts);
    const std::string kind = deck.GetString("solver.kind", "barnes_hut");
    m_opts.theta = deck.GetDouble("solver.theta", 0.5);
    const bool bhOrDirect = kind == "direct" || kind == "barnes_hut" || kind == "bh";
    if (kind == "direct") {
        m_opts.theta = 0.0;  // every node opens: the exact pair sum
    } else if (!bhOrDirect) {
        warn("solver.kind = \"" + kind + "\" runs as Barnes-Hut (the reference also falls back to it)");
    }
    m_block = deck.GetString("time.scheme", "global") == "block" && bhOrDirect;
    // solver.mac / solver.alpha (DeckSim.cpp:41-42): the relative test runs
    // on the per-particle walk (Barnes-Hut only; direct opens everything).
    if (kind != "direct" && deck.GetString("solver.mac", "geometric") == "relative") m_opts.mac = NGRAV_MAC_RELATIVE;
    m_alpha = deck.GetDouble("solver.alpha", 0.001);
    m_spline = deck.GetString("softening.kind", "plummer") == "spline";  // DeckSim.cpp:61-62
    m_opts.leaf_capacity = deck.GetInt("solver.leaf_capacity", 8);
    m_opts.quadrupole = deck.GetBool("solver.quadrupole", true) ? 1 : 0;
    m_opts.precision = deck.GetString("precision.mode", "split") == "plain" ? NGRAV_PRECISION_PLAIN
                                                                            : NGRAV_PRECISION_SPLIT;

    m_scenarioType = deck.GetString("scenario.type", "plummer");
    m_params.n = deck.GetInt("scenario.n", 2000);
    m_params.seed = (uint32_t)deck.GetInt("scenario.seed", 1);
    m_params.icFile = deck.GetString("scenario.ic_file", "");

    // A scenario carries tuned G / softening / dt; the deck overrides each
    // only when it sets the key (DeckSim.cpp:53-62, :76-84).
    m_deckHasG = deck.Has("sim.G");
    m_deckHasEps = deck.Has("softening.eps");
    m_deckHasDt = deck.Has("time.dt");
    m_deckG = deck.GetDouble("sim.G", 1.0);
    m_deckEps = deck.GetDouble("softening.eps", 0.05);
    m_deckDt = deck.GetDouble("time.dt", 1e-3);
    LoadScenario();
}

void DeckSim::LoadScenario() {
    bool fellBack = false;
    Scenario sc = BuildScenario(m_scenarioType, m_params, &fellBack);
    if (fellBack) {
        m_warnings.push_back("scenario.type = \"" + m_scenarioType + "\" is not available; Plummer sphere used");
        std::fprintf(stderr, "warning: %s\n", m_warnings.back().c_str());
    }
    m_opts.G = m_deckHasG ? m_deckG : sc.G;
    m_opts.eps = m_deckHasEps ? m_deckEps : sc.eps;
    m_dt = m_deckHasDt ? m_deckDt : sc.suggestedDt;
    m_lastDt = m_dt;
    if (!m_ctx)
        Check(ngrav_gpu_create(&m_ctx, &m_opts), "ngrav_gpu_create");
    else
        Check(ngrav_gpu_set_opts(m_ctx, &m_opts), "ngrav_gpu_set_opts");
    if (m_opts.mac == NGRAV_MAC_RELATIVE) Check(ngrav_gpu_set_mac_alpha(m_ctx, m_alpha), "ngrav_gpu_set_mac_alpha");
    Check(ngrav_gpu_set_softening(m_ctx, m_spline ? NGRAV_SOFTENING_SPLINE : NGRAV_SOFTENING_PLUMMER),
          "ngrav_gpu_set_softening");
    m_rungMax = 0;
    const State& s = sc.state;
    m_n = (long long)s.Count();
    Check(ngrav_gpu_set_particles(m_ctx, m_n, s.x.data(), s.y.data(), s.z.data(), s.vx.data(), s.vy.data(),
                                  s.vz.data(), s.m.data()),
          "ngrav_gpu_set_particles");
    m_time = 0.0;
    m_step = 0;
    ngrav_gpu_diag d;
    Check(ngrav_gpu_diagnostics(m_ctx, 0, &d), "ngrav_gpu_diagnostics");
    m_energy0 = d.energy;
    m_lmag0 = std::sqrt(d.L[0] * d.L[0] + d.L[1] * d.L[1] + d.L[2] * d.L[2]);
    Check(ngrav_gpu_prime(m_ctx), "ngrav_gpu_prime");
}

void DeckSim::Reset() { LoadScenario(); }

// System::Step per substep (System.hpp:89-107): block, else adaptive, else
// the fixed-dt KDK (batched into one call, replayed as CUDA graphs).
void DeckSim::Step(int substeps) {
    if (m_block) {
        for (int k = 0; k < substeps; ++k) {
            Check(ngrav_gpu_block_step(m_ctx, m_dt, m_eta, m_blockMaxRung, &m_rungMax), "ngrav_gpu_block_step");
            m_lastDt = m_dt;
            m_time += m_dt;
            ++m_step;
        }
        return;
    }
    if (m_adaptive) {
        for (int k = 0; k < substeps; ++k) {
            double dt = m_dt;
            Check(ngrav_gpu_adaptive_dt(m_ctx, m_eta, m_dt, &dt), "ngrav_gpu_adaptive_dt");
            Check(ngrav_gpu_step(m_ctx, 1, dt), "ngrav_gpu_step");
            m_lastDt = dt;
            m_time += dt;
            ++m_step;
        }
        return;
    }
    Check(ngrav_gpu_step(m_ctx, substeps, m_dt), "ngrav_gpu_step");
    m_lastDt = m_dt;
    m_time += m_dt * substeps;
    m_step += substeps;
}

void DeckSim::Snapshot(fw::OutputWriter& writer) {
    const size_t n = (size_t)m_n;
    m_pos.resize(n * 3);
    m_vel.resize(n * 3);
    std::vector<float>& pos = m_pos;
    std::vector<float>& vel = m_vel;
    Check(ngrav_gpu_get_frame_f32(m_ctx, pos.data(), vel.data()), "ngrav_gpu_get_frame_f32");
    writer.WriteField("pos", pos.data(), fw::NpyDtype::F4, (int)n, 3);
    writer.WriteField("vel", vel.data(), fw::NpyDtype::F4, (int)n, 3);

    ngrav_gpu_diag d;
    Check(ngrav_gpu_diagnostics(m_ctx, 0, &d), "ngrav_gpu_diagnostics");
    const double E = d.energy;
    const double lmag = std::sqrt(d.L[0] * d.L[0] + d.L[1] * d.L[1] + d.L[2] * d.L[2]);
    const double pmag = std::sqrt(d.P[0] * d.P[0] + d.P[1] * d.P[1] + d.P[2] * d.P[2]);
    writer.WriteScalar("energy", E);
    writer.WriteScalar("energy_drift_pct", (m_energy0 != 0.0) ? 100.0 * (E - m_energy0) / std::abs(m_energy0) : 0.0);
    writer.WriteScalar("L_mag", lmag);
    writer.WriteScalar("L_drift_pct", (m_lmag0 > 1e-12) ? 100.0 * (lmag - m_lmag0) / m_lmag0 : 100.0 * lmag);
    writer.WriteScalar("p_mag", pmag);
    writer.WriteScalar("com_x", d.com[0]);
    writer.WriteScalar("com_y", d.com[1]);
    writer.WriteScalar("com_z", d.com[2]);
    writer.WriteScalar("dt_last", m_lastDt);
    writer.WriteScalar("rung_max", (double)m_rungMax);  // deepest rung of the last block step
}

fw::SimInfo DeckSim::Info() const {
    fw::SimInfo info;
    info.title = m_title;
    info.dt = m_dt;
    info.substepsPerFrame = m_substepsPerFrame;
    info.frameFields = {"pos", "vel"};
    info.diagnostics = {"energy", "energy_drift_pct", "L_mag", "L_drift_pct", "p_mag",
                        "com_x",  "com_y",            "com_z", "dt_last",     "rung_max"};
    return info;
}

}  // namespace ngrav_host
