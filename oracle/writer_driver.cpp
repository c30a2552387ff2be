// writer_driver.cpp -- drives a run-directory writer through one fixed,
// deterministic three-frame run, so that two writers can be compared byte
// for byte.  Test infrastructure only.
//
// Compiled two ways:
//   -DNGRAV_WRITER_REF  against the reference's own fw::OutputWriter and
//                       fw::Deck (framework/src/OutputWriter.cpp, Deck.cpp;
//                       oracle/build_ref.sh), whose output becomes the golden
//                       fixture tests/golden/writer_run.npz;
//   otherwise           against this project's writer
//                       (opengl-physics_gb300/host/output_writer.cpp), whose
//                       output the CPU test compares with that fixture.
// Both writers take the same calls (framework/include/framework/
// OutputWriter.hpp:30-46): BeginFrame / WriteField / WriteScalar / EndFrame
// per frame, Finish once.
//
// The run covers: a title needing JSON escapes, non-round grid extents and
// dt, 2-D float32/float64 fields, a 1-D int32 field (shape (n,)), a complex64
// field, a field first written on frame 1, scalars with 10-significant-digit
// formatting, negative zero, tiny and huge magnitudes, a NaN value, and a
// diagnostics column that is never written (the writer's "nan").
//
// Usage: writer_driver <out-dir>
#ifdef NGRAV_WRITER_REF
#include "framework/Deck.hpp"
#include "framework/OutputWriter.hpp"
#else
#include "deck.hpp"
#include "simulation.hpp"
#endif

#include <cmath>
#include <cstdint>
#include <cstdio>
#include <limits>
#include <vector>

int main(int argc, char** argv) {
    if (argc != 2) {
        std::fprintf(stderr, "usage: %s <out-dir>\n", argv[0]);
        return 2;
    }
    const char* deck_text =
        "# writer fixture deck\n"
        "[sim]\nG = 1.0\n\n[time]\ndt = 0.00125\nframes = 3\nsubsteps_per_frame = 4\n";
    const fw::Deck deck = fw::Deck::FromString(deck_text, "fixture.toml");

    fw::SimInfo info;
    info.title = "Writer \"fixture\" \\ run\tA";
    info.gridNx = 5;
    info.gridNy = 3;
    info.lx = 2.5;
    info.ly = 0.333333333333;
    info.dt = 0.00125;
    info.substepsPerFrame = 4;
    info.frameFields = {"pos", "vel", "ids", "psi", "late"};
    info.diagnostics = {"energy", "energy_drift_pct", "never_written", "tiny", "huge", "negzero", "nan_value"};

    fw::OutputWriter w(argv[1], info, deck);
    const int nrow = 5;
    for (int f = 0; f < 3; ++f) {
        const long step = (long)f * 4;
        w.BeginFrame((double)step * 0.00125, step);
        std::vector<float> pos(nrow * 3), vel(nrow * 3);
        for (int i = 0; i < nrow * 3; ++i) {
            pos[i] = 0.1f * (float)(i + 1) + (float)f;
            vel[i] = -0.01f * (float)(i * i) + 0.5f * (float)f;
        }
        w.WriteField("pos", pos.data(), fw::NpyDtype::F4, nrow, 3);
        w.WriteField("vel", vel.data(), fw::NpyDtype::F4, nrow, 3);
        std::vector<int32_t> ids(7);
        for (int i = 0; i < 7; ++i) ids[i] = 100 * f - i;
        w.WriteField("ids", ids.data(), fw::NpyDtype::I4, 0, 7);
        std::vector<float> psi(2 * 4);  // complex64: interleaved re, im
        for (int i = 0; i < 8; ++i) psi[i] = (float)(i - 3) * 0.25f + (float)f;
        w.WriteField("psi", psi.data(), fw::NpyDtype::C8, 2, 2);
        if (f >= 1) {
            std::vector<double> late(3 * 2);
            for (int i = 0; i < 6; ++i) late[i] = std::sqrt((double)(i + f));
            w.WriteField("late", late.data(), fw::NpyDtype::F8, 3, 2);
        }
        w.WriteScalar("energy", -0.2462323 + 1.234567890123e-7 * f);
        w.WriteScalar("energy_drift_pct", f == 0 ? 0.0 : 1.0 / 3.0 * f);
        w.WriteScalar("tiny", 1.0e-300 * (f + 1));
        w.WriteScalar("huge", 123456789012.345 * (f + 1));
        w.WriteScalar("negzero", -0.0);
        w.WriteScalar("nan_value", std::numeric_limits<double>::quiet_NaN());
        w.WriteScalar("not_a_column", 42.0);  // not in SimInfo::diagnostics: not written
        w.EndFrame();
    }
    w.Finish();
    return 0;
}
