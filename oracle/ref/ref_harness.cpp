// ref_harness.cpp - C entry points over the reference's own functions built
// for the CPU (TEST INFRASTRUCTURE: used by the pins in tests/ and by the
// golden-vector script, never by the product).
//
// The reference's functions (cut out of its source files by ref_build.py)
// run unchanged on their own global state: tables read by its readers, the
// phantom uploaded by its initPhantom, the ring read by its read_file_ro and
// iniPanel, the Woodcock majorants built by its iniwck. Each kernel runs as
// one thread (blockDim = gridDim = 1) on one photon or pulse; its random
// numbers come from a tape of 32-bit words (see ref_prelude.h), so the
// oracle can be fed exactly the same words.
#include "ref_prelude.h"

int ref_tex_frac_bits = 0;

#include "constants.h"
int nmat_h;   // initialize.cu:6
#include "gPETInternal.h"
#include "gPET_kernals.h"
#include "externCUDA.h"
static float ref_dyn_smem[1 << 16];
using namespace std;   // detector.cu's file scope
#include "ref_sources.cpp"

namespace {

Phantom g_phantom;
std::vector<int> g_mat;
std::vector<float> g_den;
object_t* g_objects = nullptr;
object_v* g_materials = nullptr;
int g_npanels = 0;

void set_tape(const uint32_t* tape, int64_t n)
{
    cuseed[0] = curandState();
    cuseed[0].tape = tape;
    cuseed[0].n = n;
    cuseed[1] = curandState();
}

// a kernel whose thread loops `id += blockDim.x * gridDim.x` stores its state
// back to cuseed[id % NRAND] after the loop, i.e. cuseed[1] for one thread
int64_t used_after_loop() { return cuseed[1].pos; }

void copy_texture(const cudaArray* a, float* out, size_t n)
{
    std::memcpy(out, a->bits.data(), n * sizeof(float));
}

}  // namespace

extern "C" {

void ref_set_texture_fraction_bits(int bits) { ref_tex_frac_bits = bits; }

// rmater, rlamph, rcompt, rcmpsf, rphote, rrayle, rrayff (initialize.cu:279-748)
// reading <root>/data/input4gPET.*; returns nmat
int ref_load_tables(const char* root, float* eminph_out, float* emax_out)
{
    char cwd[4096];
    if (!getcwd(cwd, sizeof(cwd))) return -1;
    if (chdir(root) != 0) return -1;
    std::FILE* keep = stdout;
    stdout = std::fopen("/dev/null", "w");
    rmater(&eminph, &emax);
    rlamph();
    rcompt();
    rcmpsf();
    rphote();
    rrayle();
    rrayff();
    std::fclose(stdout);
    stdout = keep;
    if (chdir(cwd) != 0) return -1;
    *eminph_out = eminph;
    *emax_out = emax;
    return nmat_h;
}

// host tables and scalars after ref_load_tables
int ref_get_table(int which, float* out, int64_t cap)
{
    struct T { const float* p; int64_t n; };
    const T t[] = {{lamph_h, NLAPH * MAXMAT}, {compt_h, NCMPT * MAXMAT}, {phote_h, NPHTE * MAXMAT},
                   {rayle_h, NRAYL * MAXMAT}, {mucmpt_h, NCPCM * NECM * MAXMAT}, {murayl_h, NCPRL * NERL * MAXMAT},
                   {elaph_h, NLAPH}, {ecmpt_h, NCMPT}, {ephte_h, NPHTE}, {erayl_h, NRAYL}};
    if (which < 0 || which >= (int)(sizeof(t) / sizeof(t[0])) || cap < t[which].n) return -1;
    std::memcpy(out, t[which].p, sizeof(float) * (size_t)t[which].n);
    return (int)t[which].n;
}

// idleph, idlecp, idlepe, idlerl, idcpcm, idecm, idcprl, iderl (the device constants)
void ref_get_scalars(float out[8])
{
    const float v[8] = {idleph, idlecp, idlepe, idlerl, idcpcm, idecm, idcprl, iderl};
    std::memcpy(out, v, sizeof(v));
}

// initPhantom (initialize.cu:831-884) and the phantom's iniwck (:773-829)
int ref_set_phantom(const int32_t* mat, const float* den, int nx, int ny, int nz, const float d[3],
                    const float off[3], float eabsph_ev)
{
    const size_t n = (size_t)nx * ny * nz;
    g_mat.assign(mat, mat + n);
    g_den.assign(den, den + n);
    g_phantom.mat = g_mat.data();
    g_phantom.dens = g_den.data();
    g_phantom.Unxvox = nx; g_phantom.Unyvox = ny; g_phantom.Unzvox = nz;
    g_phantom.dx = d[0]; g_phantom.dy = d[1]; g_phantom.dz = d[2];
    g_phantom.Offsetx = off[0]; g_phantom.Offsety = off[1]; g_phantom.Offsetz = off[2];
    g_phantom.Sizex = nx * d[0]; g_phantom.Sizey = ny * d[1]; g_phantom.Sizez = nz * d[2];
    std::FILE* keep = stdout;
    stdout = std::fopen("/dev/null", "w");
    initPhantom(g_phantom);
    eabsph_h = eabsph_ev;
    eabsph = eabsph_ev;
    iniwck(eminph, emax, g_phantom);
    std::fclose(stdout);
    stdout = keep;
    return 0;
}

// read_file_ro (detector.cu:64-285), iniPanel (initialize.cu:969-1224) and
// the detector's iniwck (:919-966)
int ref_set_detector(const char* geo_path)
{
    char fname[100];
    std::snprintf(fname, sizeof(fname), "%s", geo_path);
    std::FILE* keep = stdout;
    stdout = std::fopen("/dev/null", "w");
    std::streambuf* cbuf = std::cout.rdbuf();
    std::ofstream sink("/dev/null");
    std::cout.rdbuf(sink.rdbuf());
    read_file_ro(&g_objects, &g_materials, &g_npanels, fname);
    iniPanel(g_objects, g_materials, g_npanels);
    iniwck(eminph, emax, g_materials);
    std::cout.rdbuf(cbuf);
    std::fclose(stdout);
    stdout = keep;
    return g_npanels;
}

// the panels as the reference holds them: per panel 31 floats in the order of
// object_t after `panel` (lengths, module, module gap, crystal, crystal gap,
// offset, direction, unit x, y, z), then the panel id; counts moduleNy,
// moduleN, crystalNy, crystalN; the two materials and densities
int ref_get_panels(float* out, int cap, int32_t counts[4], int32_t mat[2], float den[2])
{
    if (cap < g_npanels) return -1;
    for (int i = 0; i < g_npanels; ++i) {
        const object_t& o = g_objects[i];
        const float v[31] = {o.lengthx, o.lengthy, o.lengthz, o.MODx, o.MODy, o.MODz, o.Mspacex, o.Mspacey,
                             o.Mspacez, o.LSOx, o.LSOy, o.LSOz, o.spacex, o.spacey, o.spacez, o.offsetx,
                             o.offsety, o.offsetz, o.directionx, o.directiony, o.directionz, o.UniXx, o.UniXy,
                             o.UniXz, o.UniYx, o.UniYy, o.UniYz, o.UniZx, o.UniZy, o.UniZz, (float)o.panel};
        std::memcpy(out + 31 * (size_t)i, v, sizeof(v));
    }
    counts[0] = moduleNy; counts[1] = moduleN; counts[2] = crystalNy; counts[3] = crystalN;
    mat[0] = g_materials[0].material; mat[1] = g_materials[1].material;
    den[0] = g_materials[0].density; den[1] = g_materials[1].density;
    return g_npanels;
}

// quadratic surfaces of crystalSearch (main.cu:144-156 loads them the same way)
void ref_set_surfaces(int n, const float* coef10)
{
    Nsurface_d = n;
    std::memcpy(surface_d, coef10, sizeof(float) * 10 * (size_t)n);
}

// the Woodcock majorant texture (which 0: phantom, 1: detector), its first
// energy and inverse spacing
int ref_get_majorant(int which, float* tab, float* e0, float* ide)
{
    const cudaArray* a = which == 0 ? woock : woockde;
    if (!a) return -1;
    copy_texture(a, tab, NWCK);
    *e0 = wcke0;
    *ide = idlewk;
    return 0;
}

// photon() (gPET_kernals.cu:256-345) for one photon: in = x y z ux uy uz E,
// time in us; out as in; *used = tape words drawn
void ref_photon(const float in[7], double t_us, const uint32_t* tape, int64_t n, float out[7], double* t_out,
                int64_t* used)
{
    set_tape(tape, n);
    x_gBrachy[0] = make_float3(in[0], in[1], in[2]);
    vx_gBrachy[0] = make_float4(in[3], in[4], in[5], in[6]);
    d_time[0] = t_us;
    photon(1);
    out[0] = x_gBrachy[0].x; out[1] = x_gBrachy[0].y; out[2] = x_gBrachy[0].z;
    out[3] = vx_gBrachy[0].x; out[4] = vx_gBrachy[0].y; out[5] = vx_gBrachy[0].z; out[6] = vx_gBrachy[0].w;
    *t_out = d_time[0];
    *used = used_after_loop();
}

// photonde() (gPET_kernals.cu:839-1233) for one photon leaving the phantom:
// panel search, detector transport, adder and readout; pulses (48-byte
// Event records) into out[cap]; returns the pulse count
int ref_photonde(const float in[7], double t_us, int32_t eventid, int rdepth, int rpolicy, const uint32_t* tape,
                 int64_t n, Event* out, int cap, int64_t* used)
{
    set_tape(tape, n);
    rdepth_d = rdepth;
    rpolicy_d = rpolicy;
    x_gBrachy[0] = make_float3(in[0], in[1], in[2]);
    vx_gBrachy[0] = make_float4(in[3], in[4], in[5], in[6]);
    d_time[0] = t_us;
    d_eventid[0] = eventid;
    static std::vector<Event> ev(256);
    int counts[2] = {0, 0};
    nsstk = 0;
    photonde(ev.data(), counts, 1, 0, dens_panel, mat_panel, panelID, lengthx_panel, lengthy_panel, lengthz_panel,
             MODx_panel, MODy_panel, MODz_panel, Mspacex_panel, Mspacey_panel, Mspacez_panel, LSOx_panel,
             LSOy_panel, LSOz_panel, spacex_panel, spacey_panel, spacez_panel, offsetx_panel, offsety_panel,
             offsetz_panel, directionx_panel, directiony_panel, directionz_panel, UniXx_panel, UniXy_panel,
             UniXz_panel, UniYx_panel, UniYy_panel, UniYz_panel, UniZx_panel, UniZy_panel, UniZz_panel);
    *used = cuseed[0].pos;
    const int k = counts[0] < cap ? counts[0] : cap;
    for (int i = 0; i < k; ++i) out[i] = ev[(size_t)i];
    return counts[0];
}

// comsam, the free-electron Klein-Nishina sampler (gPET_kernals.cu:90-126)
void ref_comsam_kn(float e, const uint32_t* tape, int64_t n, float* efrac, float* cost, int64_t* used)
{
    set_tape(tape, n);
    comsam(e, &cuseed[0], efrac, cost);
    *used = cuseed[0].pos;
}

// comsam from the Compton surface and rylsam (gPET_kernals.cu:66-88, 128-146)
void ref_surface_sample(int which, float e, int matid, const uint32_t* tape, int64_t n, float* efrac, float* cost,
                        int64_t* used)
{
    set_tape(tape, n);
    *efrac = 1.0f;
    if (which == 0) comsam(e, &cuseed[0], efrac, cost, matid);
    else rylsam(e, matid, &cuseed[0], cost);
    *used = cuseed[0].pos;
}

// sampleEkPositron (gPET_kernals.cu:420-443) with the coefficients of one isotope
float ref_sample_ek(const float coef8[8], const uint32_t* tape, int64_t n, int64_t* used)
{
    set_tape(tape, n);
    float c[8];
    std::memcpy(c, coef8, sizeof(c));
    const float ek = sampleEkPositron(0, c, &cuseed[0]);
    *used = cuseed[0].pos;
    return ek;
}

// getPositionFromShape (gPET_kernals.cu:445-482)
void ref_shape(int shape, const float coef6[6], const uint32_t* tape, int64_t n, float p[3], int64_t* used)
{
    set_tape(tape, n);
    float c[6];
    std::memcpy(c, coef6, sizeof(c));
    const float3 r = getPositionFromShape(0, shape, c, &cuseed[0]);
    p[0] = r.x; p[1] = r.y; p[2] = r.z;
    *used = cuseed[0].pos;
}

// setPositronRange (gPET_kernals.cu:347-418) in the loaded phantom; v4 = the
// direction (used when usedirection) and the kinetic energy (eV)
void ref_positron_range(const float x[3], const float v4[4], int usedirection, const uint32_t* tape, int64_t n,
                        float out[3], int64_t* used)
{
    set_tape(tape, n);
    const float3 r = setPositronRange(make_float3(x[0], x[1], x[2]), make_float4(v4[0], v4[1], v4[2], v4[3]),
                                      &cuseed[0], usedirection);
    out[0] = r.x; out[1] = r.y; out[2] = r.z;
    *used = cuseed[0].pos;
}

// setPositionForPhoton (gPET_kernals.cu:563-604) for one positron record:
// optional range along its direction, then the annihilation pair; out:
// position (3) then per photon direction and energy (2 x 4)
void ref_psf_pair(const float x[3], const float v4[4], int useprange, float noncol, const uint32_t* tape, int64_t n,
                  float out[11], int64_t* used)
{
    set_tape(tape, n);
    NonAngle_d = noncol;
    x_gBrachy[0] = make_float3(x[0], x[1], x[2]);
    vx_gBrachy[0] = make_float4(v4[0], v4[1], v4[2], v4[3]);
    setPositionForPhoton(1, 0, useprange);
    out[0] = x_gBrachy[0].x; out[1] = x_gBrachy[0].y; out[2] = x_gBrachy[0].z;
    out[3] = vx_gBrachy[0].x; out[4] = vx_gBrachy[0].y; out[5] = vx_gBrachy[0].z; out[6] = vx_gBrachy[0].w;
    out[7] = vx_gBrachy[1].x; out[8] = vx_gBrachy[1].y; out[9] = vx_gBrachy[1].z; out[10] = vx_gBrachy[1].w;
    *used = used_after_loop();
}

// crystalSearch (gPET_kernals.cu:1236-1279) in panel p of the loaded ring
void ref_crystal_search(int p, const float x[3], int32_t ids[3])
{
    int m = -1, M = -1, L = -1;
    crystalSearch(make_float3(x[0], x[1], x[2]), lengthy_panel[p], lengthz_panel[p], MODy_panel[p], MODz_panel[p],
                  Mspacey_panel[p], Mspacez_panel[p], LSOy_panel[p], LSOz_panel[p], spacey_panel[p], spacez_panel[p],
                  directiony_panel[p], directionz_panel[p], &m, &M, &L);
    ids[0] = m; ids[1] = M; ids[2] = L;
}

// adder over n deposits of one photon, then readout (gPET_kernals.cu:737-813)
int ref_adder_readout(const Event* dep, int n, int depth, int policy, Event* out, int cap)
{
    std::vector<Event> ev((size_t)n + 1);
    int counts[2] = {0, 0};
    for (int i = 0; i < n; ++i) adder(counts, ev.data(), dep[i]);
    readout(counts, ev.data(), depth, policy);
    const int k = counts[1] < cap ? counts[1] : cap;
    for (int i = 0; i < k; ++i) out[i] = ev[(size_t)i];
    return counts[1];
}

// blur (gPET_kernals.cu:814-837) of one pulse
void ref_blur(Event* e, int policy, float Eref, float Rref, float slope, float sblur, const uint32_t* tape, int64_t n,
              int64_t* used)
{
    set_tape(tape, n);
    blur(1, e, policy, Eref, Rref, slope, sblur);
    *used = used_after_loop();
}

}  // extern "C"
