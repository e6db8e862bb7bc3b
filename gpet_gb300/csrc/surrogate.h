// surrogate.h - host-side glue between the run orchestration (gpet_api.cu)
// and the learned detector response (surrogate.cu).
#pragma once
#include "kernels.h"

struct gpet_ctx;
struct gpet_surrogate;

namespace gpet {

// what a surrogate is tied to: the panel geometry, detector materials and
// readout of the context it was made for
struct SurGeom {
    int32_t device;
    int32_t npanels;
    float panel0[15];             // panel 0: length, module size/gap, crystal size/gap
    float dirsign;                // local x of a panel grows outward (-1) or inward (+1)
    int32_t moduleN, crystalN, crystalNy;
    int32_t rdepth, rpolicy;
    int32_t ndetmat;
    int32_t det_mat[8];
    float det_den[8];
};

// device view of a surrogate for the routing and inference kernels
struct SurrogateDev {
    const float* params;          // fp32 parameters (biases and the panel embedding are read from here)
    const unsigned char* img;     // bf16 operand images of the five weight matrices
    const uint8_t* panel_ok;      // [npanels] 1: the panel is in the validated domain
    int32_t npanels;
    float half_y, half_z, depth;  // panel normalisation (cm)
    float dirsign;
    float e_lo, e_hi, margin;     // validated domain: entry energy (eV), distance from the panel edges (cm)
    int32_t crystalN, crystalNy, rdepth, rpolicy, moduleN;
    // crystal head: 0 one softmax over the crystals of a set (at most 64);
    // 1 a row softmax (columns [0, 32) of the set) and a column softmax
    // ([32, 64)), for grids of up to 32 x 32 crystals
    int32_t fact, crystalNz;
    // factorised head: multiplicative weights of each (energy class, row,
    // column) cell on the product of the row and column probabilities,
    // [2][32][32], fitted by the calibration (1 before it)
    const float* corr;
    float cry_pitch_y, cry_pitch_z, cry_y, cry_z;   // crystal pitch and size in y, z (module 0)
};

// defined in gpet_api.cu: the geometry a context holds (GPET_ERR_ARG when
// it has none)
int ctx_geometry(const gpet_ctx* c, SurGeom* g);
// defined in surrogate.cu
int surrogate_view(const gpet_surrogate* s, const SurGeom& g, SurrogateDev* out, const char** why);

// Split the first *q.count queue entries: those the surrogate handles go to
// the index list sidx (count *scount), the others are copied into q2 (count
// *q2.count) for the Monte Carlo detector kernel. max_n bounds the grid.
cudaError_t launch_route(const SurrogateDev& sd, const QueueDev& q, int64_t max_n, const QueueDev& q2,
                         uint32_t* sidx, unsigned long long* scount, cudaStream_t s);
// Detector response of the listed photons from the MLP: at most one pulse per
// photon, appended to P; per-simulation pulse and surrogate counts in cnt.
cudaError_t launch_surrogate(const SurrogateDev& sd, const SimDesc* sims, const QueueDev& q, const uint32_t* sidx,
                             const unsigned long long* scount, int64_t max_n, const PulseDev& P, Counters* cnt,
                             int* err, cudaStream_t s);

}  // namespace gpet
