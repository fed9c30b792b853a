// Phase-space file readers (host only): BEAMnrc .egsphsp and the IAEA format.
//
// .egsphsp (egs++/sources/egs_phsp_source/egs_phsp_source.cpp:77-160 header,
// :364-423 records): a header record "MODE0"/"MODE2", the particle and photon
// counts (int32), the maximum kinetic energy, the minimum electron kinetic
// energy and the incident-history count (float32), padded to one record; then
// per particle LATCH (bit 30 e-, bit 29 e+), E (total energy for e+-, negative
// for the first particle of an incident history), X, Y, U, V, WT (negative when
// W < 0) and, in MODE2, ZLAST.
//
// IAEA (HEN_HOUSE/iaea_phsp: header iaea_header.cpp:60-330, records
// iaea_record.cpp:145-230, file checks iaea_phsp.cpp:1024-1068, particle fetch
// :1170-1240; used by egs++/sources/iaea_phsp_source/iaea_phsp_source.cpp:77-224,
// :310-417): a text header <name>.IAEAheader of "$KEYWORD:" blocks and a binary
// <name>.IAEAphsp of fixed-length records.  A record is the particle type as a
// signed byte (1 photon, 2 e-, 3 e+, 4 neutron, 5 proton; negative when W < 0),
// the kinetic energy (float32, negative for a new history), then those of X, Y,
// Z, U, V, WEIGHT that RECORD_CONTENTS marks as stored (the others are the
// RECORD_CONSTANT values), the extra floats and the extra int32s.  W is not
// stored: it is sign * sqrt(1 - u^2 - v^2), and when u^2 + v^2 > 1 the reader
// rescales (u, v) to unit length and sets W = 0.  An extra int32 of type 1 is the
// incremental history number, which then decides what starts a new history; one
// of type 2 is the EGS LATCH.
#include <algorithm>
#include <cmath>
#include <cstdint>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <fstream>
#include <limits>
#include <sstream>
#include <string>
#include <vector>

#include "egsgpu.h"

namespace egsgpu_host {

static thread_local std::string g_host_err = "null handle";

const char *host_error() { return g_host_err.c_str(); }

namespace {

int fail(int code, const std::string &msg) {
    g_host_err = msg;
    return code;
}

bool host_little_endian() {
    const uint32_t one = 1;
    unsigned char b[4];
    std::memcpy(b, &one, 4);
    return b[0] == 1;
}

template <class T> T load(const unsigned char *p, bool swap) {
    unsigned char b[sizeof(T)];
    for (size_t i = 0; i < sizeof(T); ++i) b[i] = swap ? p[sizeof(T) - 1 - i] : p[i];
    T v;
    std::memcpy(&v, b, sizeof(T));
    return v;
}

bool file_size(const std::string &path, long long &size) {
    std::ifstream f(path, std::ios::binary | std::ios::ate);
    if (!f) return false;
    size = (long long)f.tellg();
    return true;
}

bool read_range(const std::string &path, long long offset, long long bytes, std::vector<unsigned char> &buf) {
    std::ifstream f(path, std::ios::binary);
    if (!f) return false;
    buf.resize((size_t)bytes);
    f.seekg(offset, std::ios::beg);
    return bytes == 0 || (bool)f.read((char *)buf.data(), bytes);
}

bool ends_with(const std::string &s, const std::string &t) {
    return s.size() >= t.size() && s.compare(s.size() - t.size(), t.size(), t) == 0;
}

int read_egsphsp(const std::string &path, long long first, long long count, egsgpu_phsp_info *info, float *out,
                 uint32_t *latch, unsigned char *newh) {
    long long size;
    std::vector<unsigned char> h;
    if (!file_size(path, size) || !read_range(path, 0, std::min(size, 32LL), h) || size < 25)
        return fail(EGSGPU_ERR_DATA, "cannot read phase-space file " + path);
    const std::string mode((const char *)h.data(), 5);
    const int rec = mode == "MODE0" ? 28 : (mode == "MODE2" ? 32 : 0);
    if (!rec) return fail(EGSGPU_ERR_DATA, path + ": not an egsphsp file");
    // the byte order is the one under which the particle count matches the file size
    bool swap = false;
    long long n = load<int32_t>(&h[5], false);
    if ((n + 1) * rec != size) {
        const long long ns = load<int32_t>(&h[5], true);
        if ((ns + 1) * rec != size)
            return fail(EGSGPU_ERR_DATA, path + ": the file size does not match the particle count in its header");
        swap = true;
        n = ns;
    }
    info->format = rec == 28 ? 0 : 1;
    info->has_latch = 1;
    info->n = n;
    info->photons = load<int32_t>(&h[9], swap);
    info->ekmax = load<float>(&h[13], swap);
    info->incident = load<float>(&h[21], swap);
    info->zmin = info->zmax = 0.0;
    if (count == 0) return EGSGPU_OK;
    if (first < 0 || count < 0 || first + count > n) return fail(EGSGPU_ERR_ARG, "record range outside the file");
    std::vector<unsigned char> b;
    if (!read_range(path, (first + 1) * rec, count * rec, b)) return fail(EGSGPU_ERR_DATA, path + ": truncated");
    const double rm = 0.5109989461;
    for (long long i = 0; i < count; ++i) {
        const unsigned char *r = &b[(size_t)i * rec];
        const uint32_t l = load<uint32_t>(r, swap);
        const float e = load<float>(r + 4, swap);
        const float q = (l & (1u << 30)) ? -1.0f : ((l & (1u << 29)) ? 1.0f : 0.0f);
        if (out) {
            float *o = out + 7 * i;
            const double ea = std::fabs((double)e);
            o[0] = q;
            o[1] = (float)(q != 0 ? ea - rm : ea);
            for (int k = 0; k < 5; ++k) o[2 + k] = load<float>(r + 8 + 4 * k, swap);
        }
        if (latch) latch[i] = l;
        if (newh) newh[i] = e < 0;
    }
    return EGSGPU_OK;
}

// One "$KEY:" block of an IAEA header: its lines, comments removed, blank lines skipped.
struct IaeaHeader {
    std::vector<std::pair<std::string, std::vector<std::string>>> blocks;
    const std::vector<std::string> *get(const std::string &key) const {
        for (auto &b : blocks)
            if (b.first == key) return &b.second;
        return nullptr;
    }
};

bool parse_iaea_header(const std::string &path, IaeaHeader &H) {
    std::ifstream f(path);
    if (!f) return false;
    std::stringstream ss;
    ss << f.rdbuf();
    std::string text = ss.str(), clean;
    // C and C++ comments, as the header reader strips them (utilities.cpp fget_c_string)
    for (size_t i = 0; i < text.size();) {
        if (text.compare(i, 2, "/*") == 0) {
            size_t j = text.find("*/", i + 2);
            i = j == std::string::npos ? text.size() : j + 2;
        } else if (text.compare(i, 2, "//") == 0) {
            size_t j = text.find('\n', i);
            i = j == std::string::npos ? text.size() : j;
        } else {
            clean += text[i++];
        }
    }
    std::istringstream in(clean);
    std::string line;
    while (std::getline(in, line)) {
        size_t a = line.find_first_not_of(" \t\r");
        if (a == std::string::npos) continue;
        line = line.substr(a, line.find_last_not_of(" \t\r") - a + 1);
        if (line[0] == '$') {
            size_t c = line.find(':');
            if (c != std::string::npos) {
                H.blocks.push_back({line.substr(1, c - 1), {}});
                continue;
            }
        }
        if (!H.blocks.empty()) H.blocks.back().second.push_back(line);
    }
    return true;
}

int read_iaea(const std::string &base, long long first, long long count, egsgpu_phsp_info *info, float *out,
              uint32_t *latch, unsigned char *newh) {
    const std::string hpath = base + ".IAEAheader", dpath = base + ".IAEAphsp";
    IaeaHeader H;
    if (!parse_iaea_header(hpath, H)) return fail(EGSGPU_ERR_DATA, "cannot open IAEA header " + hpath);
    auto one = [&](const char *key, double &v) {
        const auto *b = H.get(key);
        if (!b || b->empty()) return false;
        v = std::atof((*b)[0].c_str());
        return true;
    };
    const auto *rc = H.get("RECORD_CONTENTS");
    double checksum, reclen_hdr, order, nparticles, orig = 0;
    if (!rc || !one("CHECKSUM", checksum) || !one("RECORD_LENGTH", reclen_hdr) || !one("BYTE_ORDER", order) ||
        !one("PARTICLES", nparticles))
        return fail(EGSGPU_ERR_DATA, hpath + ": a mandatory keyword is missing");
    one("ORIG_HISTORIES", orig);
    int contents[9] = {0};
    for (int i = 0; i < 9 && i < (int)rc->size(); ++i) contents[i] = std::atoi((*rc)[i].c_str());
    const int nxf = contents[7], nxl = contents[8];
    if (nxf < 0 || nxl < 0 || nxf > 10 || nxl > 10 || (int)rc->size() < 9 + nxf + nxl)
        return fail(EGSGPU_ERR_DATA, hpath + ": malformed RECORD_CONTENTS");
    int ltype[10] = {0};
    for (int j = 0; j < nxl; ++j) ltype[j] = std::atoi((*rc)[9 + nxf + j].c_str());
    // constants of the quantities that are not stored, in the order X Y Z U V W WEIGHT
    double cst[7];
    for (double &c : cst) c = 32000.0;
    const auto *rk = H.get("RECORD_CONSTANT");
    for (int i = 0, k = 0; i < 7; ++i) {
        if (contents[i] > 0) continue;
        if (!rk || k >= (int)rk->size()) return fail(EGSGPU_ERR_DATA, hpath + ": missing RECORD_CONSTANT value");
        cst[i] = std::atof((*rk)[k++].c_str());
    }
    // record: type byte, energy, stored X Y Z U V WEIGHT, extra floats, extra longs (W is never stored)
    int nf = 1;
    for (int i = 0; i < 7; ++i)
        if (i != 5 && contents[i] > 0) ++nf;
    const long long rec = 1 + 4LL * (nf + nxf + nxl);
    const long long n = (long long)nparticles;
    long long size;
    if (!file_size(dpath, size)) return fail(EGSGPU_ERR_DATA, "cannot open IAEA phase-space file " + dpath);
    if ((long long)checksum != size || rec * n != size)
        return fail(EGSGPU_ERR_DATA, dpath + ": the file size does not match the record length and particle count");
    const int bo = (int)order;
    if (bo != 1234 && bo != 4321) return fail(EGSGPU_ERR_DATA, hpath + ": unknown BYTE_ORDER");
    const bool swap = (bo == 1234) != host_little_endian();
    info->format = 2;
    info->n = n;
    double nph = 0;
    info->photons = one("PHOTONS", nph) ? (long long)nph : 0;
    info->incident = orig;
    info->ekmax = 0.0;
    if (const auto *st = H.get("STATISTICAL_INFORMATION_PARTICLES")) {
        // one line per particle kind present: weight, wmin, wmax, <E>, Emin, Emax
        for (auto &l : *st) {
            std::istringstream ls(l);
            double v[6];
            if (ls >> v[0] >> v[1] >> v[2] >> v[3] >> v[4] >> v[5]) info->ekmax = std::max(info->ekmax, v[5]);
        }
    }
    info->has_latch = 0;
    for (int j = 0; j < nxl; ++j) info->has_latch |= ltype[j] == 2;
    const double nan = std::numeric_limits<double>::quiet_NaN();
    info->zmin = info->zmax = contents[2] > 0 ? nan : cst[2];
    if (count == 0) return EGSGPU_OK;
    if (first < 0 || count < 0 || first + count > n) return fail(EGSGPU_ERR_ARG, "record range outside the file");
    std::vector<unsigned char> b;
    if (!read_range(dpath, first * rec, count * rec, b)) return fail(EGSGPU_ERR_DATA, dpath + ": truncated");
    double zmin = INFINITY, zmax = -INFINITY;
    for (long long i = 0; i < count; ++i) {
        const unsigned char *r = &b[(size_t)(i * rec)];
        int type = (int)(int8_t)r[0];
        const bool wneg = type < 0;
        if (wneg) type = -type;
        if (type < 1 || type > 3)
            return fail(EGSGPU_ERR_DATA, dpath + ": record " + std::to_string(first + i) +
                                             " is not a photon, electron or positron (type " + std::to_string(type) + ")");
        const float e = load<float>(r + 1, swap);
        float v[7];
        for (int k = 0; k < 7; ++k) v[k] = (float)cst[k];
        const unsigned char *p = r + 5;
        for (int k = 0; k < 7; ++k) {
            if (k == 5 || contents[k] <= 0) continue;
            v[k] = load<float>(p, swap);
            p += 4;
        }
        p += 4 * nxf;
        uint32_t l = 0;
        int hist = e < 0;
        for (int j = 0; j < nxl; ++j, p += 4) {
            const int32_t x = load<int32_t>(p, swap);
            if (ltype[j] == 1) hist = x > 0;
            if (ltype[j] == 2) l = (uint32_t)x;
        }
        float u = v[3], vv = v[4], w = v[5];
        if (contents[5] > 0) {
            const float aux = u * u + vv * vv;   // in float, as the record reader forms it
            if ((double)aux <= 1.0) {
                w = std::sqrt((float)(1.0 - (double)aux));
            } else {
                const float s = std::sqrt(aux);
                u /= s;
                vv /= s;
                w = 0.0f;
            }
            if (wneg) w = -w;
        }
        zmin = std::min(zmin, (double)v[2]);
        zmax = std::max(zmax, (double)v[2]);
        if (out) {
            float *o = out + 7 * i;
            o[0] = type == 1 ? 0.0f : (type == 2 ? -1.0f : 1.0f);
            o[1] = std::fabs(e);
            o[2] = v[0];
            o[3] = v[1];
            o[4] = u;
            o[5] = vv;
            const float wt = std::fabs(v[6]);
            o[6] = (w < 0 || (w == 0 && wneg)) ? -wt : wt;
        }
        if (latch) latch[i] = l;
        if (newh) newh[i] = (unsigned char)hist;
    }
    info->zmin = zmin;
    info->zmax = zmax;
    return EGSGPU_OK;
}

}  // namespace
}  // namespace egsgpu_host

extern "C" int egsgpu_read_phsp(const char *path, long long first, long long count, egsgpu_phsp_info *info,
                                float *particles, uint32_t *latch, unsigned char *new_history) {
    using namespace egsgpu_host;
    if (!path || !info) return fail(EGSGPU_ERR_ARG, "egsgpu_read_phsp: null path or info");
    std::memset(info, 0, sizeof(*info));
    std::string p(path);
    for (const char *ext : {".IAEAheader", ".IAEAphsp"})
        if (ends_with(p, ext)) return read_iaea(p.substr(0, p.size() - std::strlen(ext)), first, count, info,
                                                particles, latch, new_history);
    std::ifstream probe(p + ".IAEAheader");
    if (probe) return read_iaea(p, first, count, info, particles, latch, new_history);
    return read_egsphsp(p, first, count, info, particles, latch, new_history);
}
