// output_writer.cpp -- run directory writer and the headless batch loop.
#include "deck.hpp"
#include "simulation.hpp"

#include <array>
#include <cstdint>
#include <cstdio>
#include <iomanip>
#include <sstream>
#include <stdexcept>
#include <sys/stat.h>

namespace fw {

namespace {

const char* DtypeDescr(NpyDtype d) {
    switch (d) {
        case NpyDtype::F4: return "<f4";
        case NpyDtype::F8: return "<f8";
        case NpyDtype::C8: return "<c8";
        case NpyDtype::I4: return "<i4";
    }
    return "<f4";
}

size_t DtypeSize(NpyDtype d) { return (d == NpyDtype::F8 || d == NpyDtype::C8) ? 8 : 4; }

void MakeDirs(const std::string& path) {
    std::string cur;
    for (size_t i = 0; i < path.size(); ++i) {
        cur += path[i];
        if (path[i] == '/' || i + 1 == path.size()) {
            if (cur.size() > 1) mkdir(cur.c_str(), 0755);
        }
    }
    struct stat st;
    if (stat(path.c_str(), &st) != 0 || !S_ISDIR(st.st_mode))
        throw std::runtime_error("OutputWriter: cannot create " + path);
}

// NumPy .npy v1.0: magic, version 1.0, little-endian u16 header length, an
// ASCII dict padded with spaces to a 64-byte multiple, '\n', then the data.
void WriteNpy(const std::string& path, const void* data, NpyDtype dtype, int ny, int nx) {
    std::ostringstream dict;
    dict << "{'descr': '" << DtypeDescr(dtype) << "', 'fortran_order': False, 'shape': (";
    if (ny > 0)
        dict << ny << ", " << nx;
    else
        dict << nx << ",";
    dict << "), }";
    std::string header = dict.str();
    const size_t unpadded = 10 + header.size() + 1;
    const size_t padded = (unpadded + 63) & ~size_t(63);
    header.append(padded - unpadded, ' ');
    header.push_back('\n');
    const uint16_t hlen = (uint16_t)header.size();
    std::ofstream f(path, std::ios::binary);
    if (!f) throw std::runtime_error("OutputWriter: cannot open " + path);
    const std::array<char, 8> magic{'\x93', 'N', 'U', 'M', 'P', 'Y', '\x01', '\x00'};
    f.write(magic.data(), magic.size());
    f.put((char)(hlen & 0xFF)).put((char)((hlen >> 8) & 0xFF));
    f.write(header.data(), (std::streamsize)header.size());
    const size_t count = (size_t)(ny > 0 ? ny : 1) * (size_t)nx;
    f.write(static_cast<const char*>(data), (std::streamsize)(count * DtypeSize(dtype)));
}

std::string JsonEscape(const std::string& s) {
    std::string out;
    for (char c : s) {
        switch (c) {
            case '"': out += "\\\""; break;
            case '\\': out += "\\\\"; break;
            case '\n': out += "\\n"; break;
            case '\r': out += "\\r"; break;
            case '\t': out += "\\t"; break;
            default: out += c;
        }
    }
    return out;
}

std::string FrameTag(int idx) {
    char buf[16];
    std::snprintf(buf, sizeof(buf), "%04d", idx);
    return buf;
}

}  // namespace

OutputWriter::OutputWriter(std::string outDir, const SimInfo& info, const Deck& deck)
    : m_dir(std::move(outDir)), m_info(info) {
    MakeDirs(m_dir + "/frames");
    {
        std::ofstream deckCopy(m_dir + "/deck.toml", std::ios::binary);
        deckCopy << deck.SourceText();
    }
    m_csv.open(m_dir + "/diagnostics.csv", std::ios::binary);
    if (!m_csv) throw std::runtime_error("OutputWriter: cannot open diagnostics.csv");
    m_csv << "t,step";
    for (const auto& name : m_info.diagnostics) m_csv << ',' << name;
    m_csv << '\n';
}

void OutputWriter::BeginFrame(double t, long step) {
    ++m_frameIndex;
    m_frameT = t;
    m_frameStep = step;
    m_pendingScalars.clear();
}

void OutputWriter::WriteField(std::string_view name, const void* data, NpyDtype dtype, int ny, int nx) {
    const std::string key(name);
    if (!m_fields.count(key)) m_fields[key] = FieldMeta{dtype, ny, nx};
    WriteNpy(m_dir + "/frames/" + key + "_" + FrameTag(m_frameIndex) + ".npy", data, dtype, ny, nx);
}

void OutputWriter::WriteScalar(std::string_view name, double value) { m_pendingScalars[std::string(name)] = value; }

void OutputWriter::EndFrame() {
    m_csv << std::setprecision(10) << m_frameT << ',' << m_frameStep;
    for (const auto& name : m_info.diagnostics) {
        auto it = m_pendingScalars.find(name);
        m_csv << ',';
        if (it != m_pendingScalars.end())
            m_csv << it->second;
        else
            m_csv << "nan";
    }
    m_csv << '\n';
    m_csv.flush();
}

void OutputWriter::Finish() {
    if (m_finished) return;
    m_finished = true;
    m_csv.close();
    const int frames = m_frameIndex + 1;
    std::ofstream j(m_dir + "/manifest.json", std::ios::binary);
    j << "{\n";
    j << "  \"title\": \"" << JsonEscape(m_info.title) << "\",\n";
    j << "  \"grid\": { \"nx\": " << m_info.gridNx << ", \"ny\": " << m_info.gridNy << ", \"lx\": " << m_info.lx
      << ", \"ly\": " << m_info.ly << " },\n";
    j << "  \"dt\": " << m_info.dt << ",\n";
    j << "  \"substeps_per_frame\": " << m_info.substepsPerFrame << ",\n";
    j << "  \"frames\": " << frames << ",\n";
    j << "  \"deck_file\": \"deck.toml\",\n";
    j << "  \"fields\": {";
    bool first = true;
    for (const auto& [name, meta] : m_fields) {
        j << (first ? "\n" : ",\n") << "    \"" << JsonEscape(name) << "\": { \"dtype\": \"" << DtypeDescr(meta.dtype)
          << "\", \"shape\": [" << meta.ny << ", " << meta.nx << "] }";
        first = false;
    }
    j << (first ? "" : "\n  ") << "},\n";
    j << "  \"diagnostics\": [";
    for (size_t i = 0; i < m_info.diagnostics.size(); ++i)
        j << (i ? ", " : "") << '"' << JsonEscape(m_info.diagnostics[i]) << '"';
    j << "]\n";
    j << "}\n";
}

int RunHeadless(Simulation& sim, const Deck& deck, const HeadlessOptions& opts) {
    const SimInfo info = sim.Info();
    int frames = opts.frames > 0 ? opts.frames : deck.GetInt("time.frames", 200);
    int substeps = opts.substeps > 0 ? opts.substeps : info.substepsPerFrame;
    if (frames < 1) frames = 1;
    if (substeps < 1) substeps = 1;
    OutputWriter writer(opts.outDir, info, deck);
    for (int f = 0; f < frames; ++f) {
        const long step = (long)f * substeps;
        const double t = (double)step * info.dt;
        writer.BeginFrame(t, step);
        sim.Snapshot(writer);
        writer.EndFrame();
        if (!opts.quiet) {
            std::printf("\rframe %d/%d  t=%.4f   ", f + 1, frames, t);
            std::fflush(stdout);
        }
        if (f + 1 < frames) sim.Step(substeps);
    }
    writer.Finish();
    if (!opts.quiet) std::printf("\ndone -> %s\n", opts.outDir.c_str());
    return 0;
}

}  // namespace fw
