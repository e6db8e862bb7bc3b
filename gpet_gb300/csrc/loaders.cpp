// loaders.cpp - parsers for gPET's input files, following the reference's
// fgets/fscanf sequences (file:line at each parser). Numbers are converted with
// strtof/strtol exactly as fscanf("%f")/("%d") does.
#include "loaders.hpp"

#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <fstream>
#include <sstream>

namespace gpet {

namespace {

bool slurp(const std::string& path, std::string& out)
{
    std::ifstream f(path, std::ios::binary);
    if (!f) return false;
    std::ostringstream ss;
    ss << f.rdbuf();
    out = ss.str();
    return true;
}

std::vector<std::string> split_lines(const std::string& s)
{
    std::vector<std::string> v;
    size_t a = 0;
    while (a <= s.size()) {
        size_t b = s.find('\n', a);
        if (b == std::string::npos) b = s.size();
        std::string ln = s.substr(a, b - a);
        if (!ln.empty() && ln.back() == '\r') ln.pop_back();
        v.push_back(ln);
        a = b + 1;
    }
    return v;
}

std::vector<std::string> tokens(const std::string& s)
{
    std::vector<std::string> v;
    std::istringstream is(s);
    std::string t;
    while (is >> t) v.push_back(t);
    return v;
}

// header line, then n whitespace-separated values over whole lines
struct LineReader {
    std::vector<std::string> lines;
    size_t i = 0;
    std::string err;
    void header() { ++i; }
    std::vector<std::string> values(size_t n)
    {
        std::vector<std::string> out;
        while (out.size() < n) {
            if (i >= lines.size()) { err = "unexpected end of file"; return out; }
            auto t = tokens(lines[i++]);
            out.insert(out.end(), t.begin(), t.end());
        }
        if (out.size() != n) err = "unexpected number of values";
        return out;
    }
};

float f32(const std::string& s) { return std::strtof(s.c_str(), nullptr); }
int i32(const std::string& s) { return (int)std::strtol(s.c_str(), nullptr, 10); }

}  // namespace

std::string read_config(const std::string& path, Config& c)
{
    std::string text;
    if (!slurp(path, text)) return "cannot open " + path;
    LineReader r;
    r.lines = split_lines(text);
    std::vector<std::string> v;
    r.header(); v = r.values(1); if (!r.err.empty()) return r.err; c.device = i32(v[0]);
    r.header(); v = r.values(1); c.noncol_sigma = f32(v[0]);
    r.header(); v = r.values(3); for (int k = 0; k < 3; ++k) c.pdim[k] = i32(v[k]);
    r.header(); v = r.values(3); for (int k = 0; k < 3; ++k) c.poffset[k] = f32(v[k]);
    r.header(); v = r.values(3); for (int k = 0; k < 3; ++k) c.psize[k] = f32(v[k]);
    r.header(); v = r.values(1); c.matfile = v.empty() ? "" : v[0];
    r.header(); v = r.values(1); c.denfile = v.empty() ? "" : v[0];
    r.header(); v = r.values(1); c.nparticle = v.empty() ? 0 : std::strtoll(v[0].c_str(), nullptr, 10);
    r.header(); v = r.values(1); c.usepsf = v.empty() ? 0 : i32(v[0]);
    r.header(); v = r.values(1); c.sourcefile = v.empty() ? "" : v[0];
    r.header(); v = r.values(1); c.ptype = v.empty() ? 0 : i32(v[0]);
    r.header(); v = r.values(1); c.useprange = v.empty() ? 0 : i32(v[0]);
    r.header(); v = r.values(2); if (v.size() == 2) { c.tstart = f32(v[0]); c.tend = f32(v[1]); }
    r.header(); v = r.values(4); for (size_t k = 0; k < v.size() && k < 4; ++k) c.recordsphere[k] = f32(v[k]);
    r.header(); v = r.values(1); c.eabsph = v.empty() ? 0.0f : f32(v[0]);
    r.header(); v = r.values(1); c.geofile = v.empty() ? "" : v[0];
    r.header(); v = r.values(1);
    int ns = v.empty() ? 0 : i32(v[0]);
    if (ns < 0 || ns > 5) return "number of quadratic surfaces must be 0..5 (MAXSURFACE, constants.h:21)";
    c.surfaces.clear();
    for (int k = 0; k < ns; ++k) {
        v = r.values(10);
        for (auto& t : v) c.surfaces.push_back(f32(t));
    }
    r.header(); v = r.values(2); if (v.size() == 2) { c.rdepth = i32(v[0]); c.rpolicy = i32(v[1]); }
    r.header(); v = r.values(1); c.eth = v.empty() ? 0.0f : f32(v[0]);
    r.header(); v = r.values(5);
    if (v.size() == 5) { c.blurpolicy = i32(v[0]); c.eref = f32(v[1]); c.rref = f32(v[2]); c.eslope = f32(v[3]); c.sblur = f32(v[4]); }
    r.header(); v = r.values(3);
    if (v.size() == 3) { c.dlevel = i32(v[0]); c.dtype = i32(v[1]); c.dtime = f32(v[2]); }
    r.header(); v = r.values(2); if (v.size() == 2) { c.ewin_lo = f32(v[0]); c.ewin_hi = f32(v[1]); }
    if (!r.err.empty()) return path + ": " + r.err;
    return "";
}

namespace {

// the (energy, value) blocks of one 1-D table file (rlamph etc.)
std::string read_1d(const std::string& path, int nmat, std::vector<float>& energy, std::vector<float>& vals)
{
    std::string text;
    if (!slurp(path, text)) return "cannot open " + path;
    auto lines = split_lines(text);
    size_t i = 0;
    vals.clear();
    for (int m = 0; m < nmat; ++m) {
        while (i < lines.size() && lines[i].find("ndata") == std::string::npos) ++i;
        if (i + 2 >= lines.size()) return path + ": fewer material blocks than materials";
        auto h = tokens(lines[i + 1]);
        if (h.empty()) return path + ": bad block header";
        int nd = i32(h[0]);
        if (nd != 4096) return path + ": array dimension does not match 4096";
        std::vector<float> e(nd);
        for (int k = 0; k < nd; ++k) {
            const char* p = lines[i + 3 + k].c_str();
            char* q;
            e[k] = std::strtof(p, &q);
            vals.push_back(std::strtof(q, nullptr));
        }
        energy = e;
        i += 3 + nd;
    }
    return "";
}

std::string read_surf(const std::string& path, int nmat, int& ncp, int& ne, float& dcp, float& de,
                      std::vector<float>& surf)
{
    std::string text;
    if (!slurp(path, text)) return "cannot open " + path + " (regenerate it with data/make_surfaces.py)";
    auto lines = split_lines(text);
    size_t i = 0;
    surf.clear();
    for (int m = 0; m < nmat; ++m) {
        while (i < lines.size() && lines[i].find("nCP") == std::string::npos) ++i;
        if (i + 1 >= lines.size()) return path + ": fewer surfaces than materials";
        auto h = tokens(lines[i + 1]);
        if (h.size() < 8) return path + ": bad surface header";
        ncp = i32(h[0]); ne = i32(h[4]); dcp = f32(h[3]); de = f32(h[7]);
        if (ncp != 301 || ne != 151) return path + ": surface must be 301 x 151 (NCPCM/NECM, constants.h:25-26)";
        for (int r = 0; r < ncp; ++r) {
            const char* p = lines[i + 4 + r].c_str();
            for (int c = 0; c < ne; ++c) {
                char* q;
                surf.push_back(std::strtof(p, &q));
                p = q;
            }
        }
        i += 4 + ncp;
    }
    return "";
}

// `infile >> n; infile.ignore(512,'#')` (initialize.cu:16-17, 123-125)
std::string count_then_hash(const std::string& text, long& n, std::vector<std::string>& tok)
{
    size_t a = text.find_first_not_of(" \t\r\n");
    if (a == std::string::npos) return "empty file";
    char* q;
    n = std::strtol(text.c_str() + a, &q, 10);
    size_t pos = q - text.c_str();
    size_t h = text.find('#', pos);
    size_t start = (h != std::string::npos && h - pos < 512) ? h + 1 : pos + 512;
    tok = tokens(start < text.size() ? text.substr(start) : std::string());
    return "";
}

}  // namespace

std::string read_tables(const std::string& dir, Tables& t)
{
    const std::string base = dir + "/input4gPET";
    std::string text;
    if (!slurp(base + ".matter", text)) return "cannot open " + base + ".matter";
    auto lines = split_lines(text);
    // rmater, initialize.cu:279-368: 4 header lines, then [Emin_ph, Emin, Emax]
    size_t k = 4;
    while (k < lines.size() && tokens(lines[k]).empty()) ++k;
    if (k >= lines.size()) return base + ".matter: missing energy range";
    auto e = tokens(lines[k]);
    if (e.size() < 3) return base + ".matter: bad energy range";
    t.eminph = f32(e[0]);
    t.emax = f32(e[2]);
    t.names.clear();
    for (auto& ln : lines) {
        size_t p = ln.find("MATERIAL:");
        if (p != std::string::npos) {
            std::string nm = ln.substr(p + 9);
            nm.erase(0, nm.find_first_not_of(" \t"));
            nm.erase(nm.find_last_not_of(" \t\r") + 1);
            t.names.push_back(nm);
        }
    }
    t.nmat = (int)t.names.size();
    if (t.nmat < 1 || t.nmat > 10) return base + ".matter: 1..10 materials supported (MAXMAT, constants.h:9)";
    std::string err;
    if (!(err = read_1d(base + ".lamph", t.nmat, t.energy, t.lamph)).empty()) return err;
    std::vector<float> e2;
    if (!(err = read_1d(base + ".compt", t.nmat, e2, t.compt)).empty()) return err;
    if (!(err = read_1d(base + ".phote", t.nmat, e2, t.phote)).empty()) return err;
    if (!(err = read_1d(base + ".rayle", t.nmat, e2, t.rayle)).empty()) return err;
    t.ne = (int)t.energy.size();
    if (!(err = read_surf(base + ".cmpsf", t.nmat, t.ncp_c, t.ne_c, t.dcp_c, t.de_c, t.cmpsf)).empty()) return err;
    if (!(err = read_surf(base + ".rayff", t.nmat, t.ncp_r, t.ne_r, t.dcp_r, t.de_r, t.rayff)).empty()) return err;
    // isotopes
    if (!slurp(dir + "/isotopes.txt", text)) return "cannot open " + dir + "/isotopes.txt";
    long n;
    std::vector<std::string> tok;
    count_then_hash(text, n, tok);
    if (n < 1 || (long)tok.size() < 10 * n) return dir + "/isotopes.txt: malformed";
    t.iso_halftime.resize(n); t.iso_ratio.resize(n); t.iso_coef.resize(8 * n);
    for (long i = 0; i < n; ++i) {
        t.iso_halftime[i] = f32(tok[10 * i]);
        t.iso_ratio[i] = f32(tok[10 * i + 1]);
        for (int c = 0; c < 8; ++c) t.iso_coef[8 * i + c] = f32(tok[10 * i + 2 + c]);
    }
    return "";
}

void panel_counts(const float* p, int& mny, int& mn, int& cny, int& cn)
{
    // iniPanel, initialize.cu:1074-1086 (float arithmetic)
    mny = (int)floorf(p[1] / (p[4] + p[7])) + 1;
    cny = (int)floorf(p[4] / (p[10] + p[13])) + 1;
    mn = mny * ((int)floorf(p[2] / (p[5] + p[8])) + 1);
    cn = cny * ((int)floorf(p[5] / (p[11] + p[14])) + 1);
}

std::string read_geometry(const std::string& path, Geometry& g)
{
    std::string text;
    if (!slurp(path, text)) return "cannot open " + path;
    LineReader r;
    r.lines = split_lines(text);
    std::vector<std::string> v;
    r.header(); v = r.values(1); if (!r.err.empty()) return path + ": " + r.err;
    g.npanels = i32(v[0]);
    if (g.npanels < 1 || g.npanels > kMaxPanelsHost) return path + ": 1..256 panels supported";
    r.header(); v = r.values(3); for (int k = 0; k < 3; ++k) g.axis[k] = f32(v[k]);
    r.header(); v = r.values(1); g.angle = f32(v[0]);
    // (material, density) pairs up to the separator line: two in the
    // reference's files, more for crystal regions marked by the surfaces
    r.header();
    v.clear();
    while (r.i < r.lines.size()) {
        auto t = tokens(r.lines[r.i]);
        if (t.empty()) { ++r.i; continue; }
        char* end = nullptr;
        std::strtod(t[0].c_str(), &end);
        if (end == t[0].c_str() || *end) break;   // not a number: the separator
        v.insert(v.end(), t.begin(), t.end());
        ++r.i;
    }
    if (v.size() < 4 || v.size() % 2 || v.size() / 2 > 8) return path + ": 2 to 8 (material, density) pairs expected";
    g.ndetmat = (int)(v.size() / 2);
    for (int k = 0; k < g.ndetmat; ++k) { g.det_mat[k] = i32(v[2 * k]); g.det_den[k] = f32(v[2 * k + 1]); }
    r.header();                                  // separator line
    float P[32] = {0};
    r.header(); v = r.values(1); P[30] = (float)i32(v[0]);
    const int offs[10] = {0, 3, 6, 9, 12, 18, 15, 21, 24, 27};   // len MOD Ms LSO s dir o UX UY UZ
    for (int b = 0; b < 10; ++b) {
        r.header();
        v = r.values(3);
        if (!r.err.empty()) return path + ": " + r.err;
        for (int k = 0; k < 3; ++k) P[offs[b] + k] = f32(v[k]);
    }
    g.panels.assign((size_t)g.npanels * 32, 0.0f);
    const float* rot = g.axis;
    for (int i = 0; i < g.npanels; ++i) {
        float* Q = &g.panels[(size_t)i * 32];
        std::memcpy(Q, P, sizeof(P));
        if (i == 0) continue;
        Q[30] = (float)i;
        // Rodrigues rotation by i*angle, detector.cu:246-278
        float ang = g.angle * 3.1415926535897932384626433f / 180.0f * (float)i;
        float ca = cosf(ang), sa = sinf(ang);
        for (int off : {15, 21, 24, 27}) {
            float vec[3] = {P[off], P[off + 1], P[off + 2]};
            Q[off + 0] = (1 - ca) * (vec[0] * rot[0]) * rot[0] + ca * vec[0] + sa * (rot[1] * vec[2] - rot[2] * vec[1]);
            Q[off + 1] = (1 - ca) * (vec[1] * rot[1]) * rot[1] + ca * vec[1] + sa * (rot[2] * vec[0] - rot[0] * vec[2]);
            Q[off + 2] = (1 - ca) * (vec[2] * rot[2]) * rot[2] + ca * vec[2] + sa * (rot[0] * vec[1] - rot[1] * vec[0]);
        }
    }
    panel_counts(P, g.moduleNy, g.moduleN, g.crystalNy, g.crystalN);
    return "";
}

std::string read_sources(const std::string& path, Sources& s)
{
    std::string text;
    if (!slurp(path, text)) return "cannot open " + path;
    long n;
    std::vector<std::string> tok;
    count_then_hash(text, n, tok);
    if (n < 1 || (long)tok.size() < 9 * n) return path + ": malformed source file";
    s.natom.resize(n); s.type.resize(n); s.shape.resize(n); s.coef.resize(6 * n);
    for (long i = 0; i < n; ++i) {
        s.natom[i] = (uint32_t)std::strtoul(tok[9 * i].c_str(), nullptr, 10);
        s.type[i] = i32(tok[9 * i + 1]);
        s.shape[i] = i32(tok[9 * i + 2]);
        for (int c = 0; c < 6; ++c) s.coef[6 * i + c] = f32(tok[9 * i + 3 + c]);
    }
    return "";
}

std::string read_phantom(const std::string& matfile, const std::string& denfile, int64_t n, std::vector<int32_t>& mat,
                         std::vector<float>& den)
{
    mat.resize(n);
    den.resize(n);
    FILE* f = std::fopen(matfile.c_str(), "rb");
    if (!f) return "cannot open " + matfile;
    size_t got = std::fread(mat.data(), 4, (size_t)n, f);
    std::fclose(f);
    if ((int64_t)got != n) return matfile + ": fewer voxels than the phantom dimension";
    f = std::fopen(denfile.c_str(), "rb");
    if (!f) return "cannot open " + denfile;
    got = std::fread(den.data(), 4, (size_t)n, f);
    std::fclose(f);
    if ((int64_t)got != n) return denfile + ": fewer voxels than the phantom dimension";
    return "";
}

std::string read_psf(const std::string& path, int64_t nmax, std::vector<double>& rec)
{
    FILE* f = std::fopen(path.c_str(), "rb");
    if (!f) return "cannot open " + path;
    std::fseek(f, 0, SEEK_END);
    long long bytes = std::ftell(f);
    std::fseek(f, 0, SEEK_SET);
    int64_t n = bytes / 64;
    if (nmax > 0 && nmax < n) n = nmax;   // readParticle, initialize.cu:88-92
    rec.resize((size_t)n * 8);
    size_t got = std::fread(rec.data(), 64, (size_t)n, f);
    std::fclose(f);
    if ((int64_t)got != n) return path + ": short read";
    return "";
}

}  // namespace gpet
