// output_writer.cpp -- the run directory of a headless deck run and the
// batch loop that fills it.
//
// The directory is the drop-in contract with the reference's Python tools
// (the layout of framework/src/OutputWriter.cpp:38-167), so its bytes are
// fixed; the code below produces them from this format description:
//   deck.toml          the deck's source text, verbatim
//   frames/<f>_NNNN.npy  one NumPy v1.0 file per field per frame, NNNN the
//                      zero-padded frame index: "\x93NUMPY", bytes 1 and 0,
//                      a little-endian u16 header length, then the header
//                      "{'descr': '<f4', 'fortran_order': False, 'shape':
//                      (ny, nx), }" (or "(nx,)" for ny = 0) padded with
//                      spaces and a final '\n' so the data starts at a
//                      multiple of 64 bytes, then the raw row-major data
//   diagnostics.csv    "t,step,<diagnostics...>", then one row per frame:
//                      t and every scalar as %.10g, the step as an integer,
//                      "nan" for a column the frame did not write
//   manifest.json      two-space-indented JSON: title, grid {nx, ny, lx,
//                      ly}, dt, substeps_per_frame, frames, deck_file, the
//                      fields in name order with the dtype and [ny, nx] of
//                      their first write, and the diagnostics names;
//                      doubles as %g, strings with ", \, \n, \r and \t
//                      escaped
// tests/test_host_cli.py checks every byte against the reference's own
// writer on a fixed run (tests/golden/writer_run.npz).
#include "deck.hpp"
#include "simulation.hpp"

#include <algorithm>
#include <cerrno>
#include <cmath>
#include <cstdint>
#include <cstdio>
#include <cstring>
#include <stdexcept>
#include <string>
#include <sys/stat.h>

namespace fw {

namespace {

struct DtypeSpec {
    const char* descr;   // NumPy type string
    size_t bytes;        // bytes per element
};

DtypeSpec Spec(NpyDtype d) {
    switch (d) {
        case NpyDtype::F8: return {"<f8", 8};
        case NpyDtype::C8: return {"<c8", 8};
        case NpyDtype::I4: return {"<i4", 4};
        case NpyDtype::F4: break;
    }
    return {"<f4", 4};
}

// printf's %.<sig>g, the formatting of every floating-point value written.
std::string Fmt(double v, int sig) {
    char buf[64];
    std::snprintf(buf, sizeof(buf), "%.*g", sig, v);
    return buf;
}

std::string JsonString(const std::string& s) {
    std::string q = "\"";
    for (const char c : s) {
        const char* esc = c == '"' ? "\\\"" : c == '\\' ? "\\\\" : c == '\n' ? "\\n" : c == '\r' ? "\\r"
                                                                                     : c == '\t' ? "\\t" : nullptr;
        if (esc)
            q += esc;
        else
            q += c;
    }
    return q + "\"";
}

// mkdir -p
void EnsureDir(const std::string& path) {
    for (size_t pos = 1; pos <= path.size(); ++pos) {
        if (pos == path.size() || path[pos] == '/') {
            const std::string prefix = path.substr(0, pos);
            if (mkdir(prefix.c_str(), 0755) != 0 && errno != EEXIST)
                throw std::runtime_error("OutputWriter: cannot create " + prefix);
        }
    }
    struct stat st;
    if (stat(path.c_str(), &st) != 0 || !S_ISDIR(st.st_mode))
        throw std::runtime_error("OutputWriter: cannot create " + path);
}

// Writes `parts` back to back into a new file at `path`.
void WriteFile(const std::string& path, std::initializer_list<std::pair<const void*, size_t>> parts) {
    FILE* f = std::fopen(path.c_str(), "wb");
    if (!f) throw std::runtime_error("OutputWriter: cannot open " + path);
    bool ok = true;
    for (const auto& p : parts) ok = ok && (p.second == 0 || std::fwrite(p.first, 1, p.second, f) == p.second);
    ok = (std::fclose(f) == 0) && ok;
    if (!ok) throw std::runtime_error("OutputWriter: cannot write " + path);
}

// Everything of a .npy file before its data.
std::string NpyPreamble(NpyDtype d, int ny, int nx) {
    const std::string shape =
        ny > 0 ? "(" + std::to_string(ny) + ", " + std::to_string(nx) + ")" : "(" + std::to_string(nx) + ",)";
    const std::string dict =
        std::string("{'descr': '") + Spec(d).descr + "', 'fortran_order': False, 'shape': " + shape + ", }";
    const size_t fixed = 10;                                 // magic, version, header length
    const size_t total = (fixed + dict.size() + 1 + 63) / 64 * 64;
    const size_t hlen = total - fixed;
    std::string out = "\x93NUMPY";
    out += '\x01';
    out += '\x00';
    out += (char)(hlen & 0xFF);
    out += (char)((hlen >> 8) & 0xFF);
    out += dict;
    out.append(total - out.size() - 1, ' ');
    out += '\n';
    return out;
}

}  // namespace

OutputWriter::OutputWriter(std::string outDir, const SimInfo& info, const Deck& deck)
    : m_dir(std::move(outDir)), m_info(info) {
    EnsureDir(m_dir + "/frames");
    const std::string& src = deck.SourceText();
    WriteFile(m_dir + "/deck.toml", {{src.data(), src.size()}});
    for (size_t k = 0; k < m_info.diagnostics.size(); ++k) m_column.emplace(m_info.diagnostics[k], k);
    m_csv = std::fopen((m_dir + "/diagnostics.csv").c_str(), "wb");
    if (!m_csv) throw std::runtime_error("OutputWriter: cannot open diagnostics.csv");
    std::string header = "t,step";
    for (const auto& name : m_info.diagnostics) header += "," + name;
    header += "\n";
    std::fputs(header.c_str(), m_csv);
}

OutputWriter::~OutputWriter() {
    if (m_csv) std::fclose(m_csv);
}

void OutputWriter::BeginFrame(double t, long step) {
    ++m_frames;
    m_t = t;
    m_step = step;
    m_row.assign(m_info.diagnostics.size(), std::nan(""));
}

void OutputWriter::WriteField(std::string_view name, const void* data, NpyDtype dtype, int ny, int nx) {
    const std::string key(name);
    const auto seen = std::find_if(m_fieldLog.begin(), m_fieldLog.end(),
                                   [&](const FieldShape& s) { return s.name == key; });
    if (seen == m_fieldLog.end()) m_fieldLog.push_back(FieldShape{key, dtype, ny, nx});
    char tag[16];
    std::snprintf(tag, sizeof(tag), "_%04d.npy", m_frames - 1);
    const std::string pre = NpyPreamble(dtype, ny, nx);
    const size_t bytes = (size_t)std::max(ny, 1) * (size_t)nx * Spec(dtype).bytes;
    WriteFile(m_dir + "/frames/" + key + tag, {{pre.data(), pre.size()}, {data, bytes}});
}

void OutputWriter::WriteScalar(std::string_view name, double value) {
    const auto it = m_column.find(std::string(name));
    if (it != m_column.end() && it->second < m_row.size()) m_row[it->second] = value;
}

void OutputWriter::EndFrame() {
    std::string line = Fmt(m_t, 10) + "," + std::to_string(m_step);
    for (const double v : m_row) line += "," + Fmt(v, 10);
    line += "\n";
    std::fputs(line.c_str(), m_csv);
    std::fflush(m_csv);  // a run that dies keeps the rows written so far
}

void OutputWriter::Finish() {
    if (!m_csv) return;
    std::fclose(m_csv);
    m_csv = nullptr;
    std::vector<FieldShape> fields = m_fieldLog;
    std::sort(fields.begin(), fields.end(), [](const FieldShape& a, const FieldShape& b) { return a.name < b.name; });
    std::string j = "{\n";
    j += "  \"title\": " + JsonString(m_info.title) + ",\n";
    j += "  \"grid\": { \"nx\": " + std::to_string(m_info.gridNx) + ", \"ny\": " + std::to_string(m_info.gridNy) +
         ", \"lx\": " + Fmt(m_info.lx, 6) + ", \"ly\": " + Fmt(m_info.ly, 6) + " },\n";
    j += "  \"dt\": " + Fmt(m_info.dt, 6) + ",\n";
    j += "  \"substeps_per_frame\": " + std::to_string(m_info.substepsPerFrame) + ",\n";
    j += "  \"frames\": " + std::to_string(m_frames) + ",\n";
    j += "  \"deck_file\": \"deck.toml\",\n";
    j += "  \"fields\": {";
    for (size_t k = 0; k < fields.size(); ++k) {
        const FieldShape& s = fields[k];
        j += (k ? ",\n    " : "\n    ") + JsonString(s.name) + ": { \"dtype\": \"" + Spec(s.dtype).descr +
             "\", \"shape\": [" + std::to_string(s.ny) + ", " + std::to_string(s.nx) + "] }";
    }
    j += fields.empty() ? "},\n" : "\n  },\n";
    j += "  \"diagnostics\": [";
    for (size_t k = 0; k < m_info.diagnostics.size(); ++k) j += (k ? ", " : "") + JsonString(m_info.diagnostics[k]);
    j += "]\n}\n";
    WriteFile(m_dir + "/manifest.json", {{j.data(), j.size()}});
}

int RunHeadless(Simulation& sim, const Deck& deck, const HeadlessOptions& opts) {
    const SimInfo info = sim.Info();
    const int frames = std::max(1, opts.frames > 0 ? opts.frames : deck.GetInt("time.frames", 200));
    const int substeps = std::max(1, opts.substeps > 0 ? opts.substeps : info.substepsPerFrame);
    OutputWriter out(opts.outDir, info, deck);
    long step = 0;
    for (int f = 1;; ++f) {
        out.BeginFrame((double)step * info.dt, step);
        sim.Snapshot(out);
        out.EndFrame();
        if (!opts.quiet) std::fprintf(stderr, "\r[nbody_gb300] frame %d of %d, step %ld", f, frames, step);
        if (f == frames) break;
        sim.Step(substeps);
        step += substeps;
    }
    out.Finish();
    if (!opts.quiet) std::fprintf(stderr, "\n[nbody_gb300] %d frames written to %s\n", frames, opts.outDir.c_str());
    return 0;
}

}  // namespace fw
