// loaders.hpp - parsers for gPET's input files (host side of the drop-in
// surface). Each parser follows the reference's fgets/fscanf sequence: a
// header line is skipped, then the expected number of values is read.
#pragma once
#include <cstdint>
#include <string>
#include <vector>

namespace gpet {

constexpr int kMaxPanelsHost = 256;

struct Config {                      // input_PET.in, main.cu:50-182
    int device = 0;
    float noncol_sigma = 0.0f;
    int pdim[3] = {0, 0, 0};
    float poffset[3] = {0, 0, 0}, psize[3] = {0, 0, 0};
    std::string matfile, denfile;
    long long nparticle = 0;
    int usepsf = 0;
    std::string sourcefile;
    int ptype = 0, useprange = 0;
    float tstart = 0.0f, tend = 1.0f;
    float recordsphere[4] = {0, 0, 0, 0};
    float eabsph = 0.0f;
    std::string geofile;
    std::vector<float> surfaces;     // 10 per surface
    int rdepth = 2, rpolicy = 1;
    float eth = 0.0f;
    int blurpolicy = 1;
    float eref = 0, rref = 0, eslope = 0, sblur = 0;
    int dlevel = 3, dtype = 0;
    float dtime = 0.0f;
    float ewin_lo = 0, ewin_hi = 0;
};

struct Tables {                      // initialize.cu:279-748
    std::vector<std::string> names;
    float eminph = 0, emax = 0;
    int nmat = 0, ne = 0;
    std::vector<float> energy;       // [ne]
    std::vector<float> lamph, compt, phote, rayle;   // [nmat][ne]
    int ncp_c = 0, ne_c = 0;
    float dcp_c = 0, de_c = 0;
    std::vector<float> cmpsf;        // [nmat][ncp][ne]
    int ncp_r = 0, ne_r = 0;
    float dcp_r = 0, de_r = 0;
    std::vector<float> rayff;
    // isotopes.txt (loadIsotopes, initialize.cu:10-31)
    std::vector<float> iso_halftime, iso_ratio, iso_coef;   // coef [n][8]
};

struct Geometry {                    // detector.cu:64-285
    int npanels = 0;
    float axis[3] = {0, 0, 1};
    float angle = 0;
    // detector materials: 0 crystal, 1 gap (the reference's two,
    // detector.cu:110-118), 2.. crystal materials of the regions that the
    // quadratic surfaces 0.. mark (more (material, density) pairs in the file)
    int ndetmat = 2;
    int det_mat[8] = {0, 0, 0, 0, 0, 0, 0, 0};
    float det_den[8] = {0, 0, 0, 0, 0, 0, 0, 0};
    std::vector<float> panels;       // [npanels][32]
    int moduleNy = 0, moduleN = 0, crystalNy = 0, crystalN = 0;
};

struct Sources {                     // initialize.cu:116-144
    std::vector<uint32_t> natom;
    std::vector<int32_t> type, shape;
    std::vector<float> coef;         // [n][6]
};

// all return "" on success or an error message
std::string read_config(const std::string& path, Config& c);
std::string read_tables(const std::string& data_dir, Tables& t);
std::string read_geometry(const std::string& path, Geometry& g);
std::string read_sources(const std::string& path, Sources& s);
std::string read_phantom(const std::string& matfile, const std::string& denfile, int64_t n, std::vector<int32_t>& mat,
                         std::vector<float>& den);
std::string read_psf(const std::string& path, int64_t nmax, std::vector<double>& rec);
void panel_counts(const float* p, int& mny, int& mn, int& cny, int& cn);

}  // namespace gpet
