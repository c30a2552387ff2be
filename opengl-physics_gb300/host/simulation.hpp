// simulation.hpp -- the batch-run contract: fw::Simulation, its static
// SimInfo, the OutputWriter that records a run, and RunHeadless.
//
// Mirrors framework/include/framework/{Simulation,OutputWriter,
// HeadlessRunner}.hpp of the reference (Simulation.hpp:14-66,
// OutputWriter.hpp:30-62, HeadlessRunner.hpp:12-20) for the headless path:
// Configure -> loop { Snapshot; Step } -> manifest.  The interactive/GL hooks
// (Render, OnViewInput, OnKey) have no counterpart: there is no graphics
// stack on this system.
#pragma once

#include <cstdio>
#include <string>
#include <string_view>
#include <unordered_map>
#include <vector>

namespace fw {

class Deck;
class OutputWriter;

struct SimInfo {
    std::string title;
    int gridNx = 0;
    int gridNy = 0;
    double lx = 0.0;
    double ly = 0.0;
    double dt = 0.0;
    int substepsPerFrame = 1;
    std::vector<std::string> frameFields;   // .npy fields written per frame
    std::vector<std::string> diagnostics;   // CSV columns after "t,step"
};

class Simulation {
public:
    virtual ~Simulation() = default;
    virtual void Configure(const Deck& deck) = 0;
    virtual void Reset() = 0;
    virtual void Step(int substeps) = 0;
    virtual void Snapshot(OutputWriter& writer) = 0;
    virtual SimInfo Info() const = 0;
};

// NumPy .npy element types (OutputWriter.hpp:15-17).
enum class NpyDtype { F4, F8, C8, I4 };

// <dir>/deck.toml, <dir>/manifest.json, <dir>/diagnostics.csv and
// <dir>/frames/<field>_NNNN.npy, byte-compatible with the reference's writer
// (the format of framework/src/OutputWriter.cpp:38-167; output_writer.cpp
// states it).  Per frame: BeginFrame, then WriteField / WriteScalar, then
// EndFrame; Finish once at the end writes the manifest.
class OutputWriter {
public:
    OutputWriter(std::string outDir, const SimInfo& info, const Deck& deck);
    ~OutputWriter();
    OutputWriter(const OutputWriter&) = delete;
    OutputWriter& operator=(const OutputWriter&) = delete;

    void BeginFrame(double t, long step);
    void WriteField(std::string_view name, const void* data, NpyDtype dtype, int ny, int nx);
    void WriteScalar(std::string_view name, double value);
    void EndFrame();
    void Finish();
    // Index of the frame begun last (the reference's accessor: frames - 1).
    int FramesWritten() const { return m_frames - 1; }

private:
    struct FieldShape {             // a field's dtype and shape at its first write
        std::string name;
        NpyDtype dtype;
        int ny, nx;
    };
    std::string m_dir;
    SimInfo m_info;
    std::FILE* m_csv = nullptr;
    std::unordered_map<std::string, size_t> m_column;  // diagnostics name -> CSV column
    std::vector<FieldShape> m_fieldLog;                // in order of first write
    std::vector<double> m_row;                         // this frame's scalars (NaN: not written)
    int m_frames = 0;                                  // frames begun
    double m_t = 0.0;
    long m_step = 0;
};

struct HeadlessOptions {
    std::string outDir;
    int frames = 0;     // 0 -> deck time.frames (default 200)
    int substeps = 0;   // 0 -> SimInfo::substepsPerFrame
    bool quiet = false;
};

// framework/src/HeadlessRunner.cpp:11-41: write a frame, advance, repeat;
// then the manifest.  Returns 0.
int RunHeadless(Simulation& sim, const Deck& deck, const HeadlessOptions& opts);

}  // namespace fw
