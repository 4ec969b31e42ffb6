// MD force evaluation (the ZCalc / Cheby::Force_all path) on the device.
//
// Reference: ZCalc (src/functions.C:815-891), Cheby::Force_all (src/Cheby.C:1731-2021),
// Force_3B (src/Cheby.C:2024-2300), Force_4B (src/Cheby.C:2303-2675).
//
// The clusters are the ones the design-matrix path enumerates (same neighbour
// convention and cut-off tests); the 2-body list additionally keeps r <= s_min
// (smoothed basis plus the cubic penalty).  Per cluster the coefficients are
// contracted as one dense tensor over the canonical pair slots, so energy and all
// edge derivatives come out of a single depth-first pass.
#pragma once
#include "kernels.h"

namespace cgd {

// Per-frame scalars written by the force pass:
//   [0] potential energy, [1] scalar virial pressure term (PRESSURE_XYZ / 3V),
//   [2..10] virial tensor / V, row-major xx xy xz yx yy yz zx zy zz.
constexpr int MD_NSCALAR = 11;

struct MdDev {
    const double* c2;       // [npairs * order2]  coefficient of T_{n+1} of pair type
    const double* C3;       // [ntypes3 * O3^3]   dense, canonical slots, slot 0 most significant
    const double* C4;       // [ntypes4 * O4^6]
    const float* C3f;       // FP32 copies (contraction precision 1)
    const float* C4f;
    const double* eoff;     // [natmtyp] per-atom energy offsets, or null
    double pen_dist, pen_scale;   // 2-body penalty (src/chimes_md.C:1747-1748 defaults)
    int coulomb;            // Ewald sums with the charges qtype (electron units)
    double qtype[10];       // charge of each atom type
};

// Ewald Coulomb forces, energy and virial of MD frames (ZCalc_Ewald, src/Ewald.C:28-426),
// added to the raw (pre-normalisation) scalars; S holds md_ewald_scratch_bytes.
size_t md_ewald_scratch_bytes(int nframes, int kmax_max);
void launch_md_ewald(int nframes, int nreal, int kmax_max, const ModelDev& M, const MdDev& D, const FramesDev& F,
                     void* S, double* Fo, double* So, cudaStream_t st);

// Clusters grouped by key = frame * ntypes + type for the contraction kernels: the
// order inside a group is not fixed (the forces are accumulated with atomics).
struct MdBuckets {
    int nkeys, ntypes;
    int64_t* start;       // [nkeys + 1] first grouped cluster of each key
    int* tile_ofs;        // [nkeys + 1] first MDC tile (block) of each key
    int* cursor;          // [nkeys] fill cursors
    int* val;             // [n] global cluster indices, grouped
};
constexpr int MDC_TILE = 64;    // clusters per contraction block

// Group n clusters of a batch (cluster frame offsets cfo) by (frame, type).
void launch_md_bucket(int64_t n, int nframes, const int64_t* cfo, const int* type, const MdBuckets& B,
                      cudaStream_t st);

// Orders with an unrolled contraction kernel; others use the generic kernel.
bool md_fast_order(int nbody, int order);

void launch_md2(const ModelDev& M, const MdDev& D, const FramesDev& F, const NeighDev& NB, double* Fo, double* So,
                cudaStream_t st, int prec = 0);
// Clusters of one body count, one block per tile of a (frame, type) group; max_tiles
// bounds the number of tiles (n / MDC_TILE + nkeys).
void launch_mdc(int nbody, int prec, int order, int64_t max_tiles, const ModelDev& M, const MdDev& D,
                const FramesDev& F, const ClusterSet& CS, const MdBuckets& B, double* Fo, double* So,
                cudaStream_t st);
void launch_md_finalize(int nframes, const ModelDev& M, const MdDev& D, const FramesDev& F, double* So,
                        cudaStream_t st);
// List reuse: per-step exact filter of skin-enumerated clusters (type_out -1 when
// out of range), and the largest squared displacement since the lists were built.
void launch_md_filter(int nbody, const ModelDev& M, const FramesDev& F, const ClusterSet& CS, const int64_t* cfo,
                      int64_t n, int* type_out, cudaStream_t st);
void launch_md_maxdisp(const double* x, const double* xref, int64_t n, unsigned long long* out, cudaStream_t st);

// Velocity Verlet (CONSTRAINT::UPDATE_COORDS / UPDATE_VELOCS_HALF_1 / _2,
// src/ClassDefs.C:870-900, 1088-1157) over every real atom of the batch.
// drift: x += v dt + a dt^2 / 2, v += a dt / 2.   kick: a = F / m, v += a dt / 2,
// kinetic energy per frame into ke[f] (when ke is not null).  first (per frame, may
// be null): frames at their step 0, which neither drift nor kick.
void launch_md_drift(int64_t natoms, const FramesDev& F, const unsigned char* first, double* xyz, double* v,
                     const double* acc, double dt, cudaStream_t st);
void launch_md_kick(int nframes, const FramesDev& F, const double* Fo, const double* inv_mass_type,
                    const double* mass_type, double* acc, double* v, double dt, int half, const unsigned char* first,
                    double* ke, cudaStream_t st);
// Thermostats and barostats (NVT-MTK, NVT-BEREND, NPT-BEREND(-ANISO), NPT-MTK):
// per-frame state of MD_TH_STRIDE doubles, CONSTRAINT's members
// (src/ClassDefs.C:479-520): thermostat velocity zeta, force, position, inertia Q,
// N_DOF kB T, the kinetic energy of the step's incoming velocities, zeta / force at
// the step's start; barostat position, velocity, force, inertia W and their values
// at the step's start, the volume after the step's coordinate update and the
// barostat's box scale.
enum {
    TH_ZETA = 0, TH_FORCE, TH_POSIT, TH_Q, TH_NDOFKT, TH_KCUR, TH_ZETA0, TH_FORCE0,
    TH_BPOS, TH_BVEL, TH_BFORCE, TH_W, TH_BVEL0, TH_BFORCE0, TH_VOL, TH_NDOF, TH_NDOF1KT, TH_SCALE,
    TH_POSIT0, TH_BPOS0, TH_VOL0, TH_VSCALE, TH_TAVG
};
constexpr int MD_TH_STRIDE = 23;
// NVT-SCALE (src/chimes_md.C:1086-1094, CONSTRAINT::SCALE_VELOCITIES
// src/ClassDefs.C:1447-1469): after step `step`, the temperature of v joins a running
// sum; every freq-th step v *= sqrt(T0 / mean) and the sum restarts.
void launch_md_vscale(int nframes, const FramesDev& F, const double* mass_type, double* v, double* th, int step,
                      int freq, double T0, double kb, cudaStream_t st);
// NPT-BEREND / NPT-BEREND-ANISO coordinate step (one block per frame): drift and
// half kick, then x and the orthorhombic cell scaled by (1 - dt/kp (P0 - P))^(1/3)
// with P from so_prev (the last force call's PRESSURE_XYZ or tensor diagonal) plus
// the kinetic term of v(t).  box is the frames' device cell array.
void launch_md_npt_berend(int nframes, const FramesDev& F, BoxDev* box, const double* mass_type, double* x,
                          double* v, const double* acc, double dt, const double* so_prev, double p0, double kp,
                          int aniso, int* bad, cudaStream_t st);
// NPT-MTK (Martyna, Tobias, Klein 1994 as CONSTRAINT does it): coordinates,
// thermostat and barostat positions, cell scale and the first velocity half; then
// the second half with the 10-step fixed point of thermostat and barostat velocity.
void launch_md_nptmtk_half1(int nframes, const FramesDev& F, BoxDev* box, const double* mass_type, double* x,
                            double* v, const double* acc, double dt, double* th, cudaStream_t st);
void launch_md_nptmtk_half2(int nframes, const FramesDev& F, const double* Fo, const double* inv_mass_type,
                            const double* mass_type, const double* so, double p0, double* acc, double* v, double dt,
                            double* th, double* ke, cudaStream_t st);
// Volume of each frame's cell into out[f].
void launch_md_volume(int nframes, const BoxDev* box, double* out, cudaStream_t st);
void launch_md_mtk_half1(int nframes, const FramesDev& F, const double* mass_type, double* x, double* v,
                         const double* acc, double dt, double* th, cudaStream_t st);
void launch_md_mtk_half2(int nframes, const FramesDev& F, const double* Fo, const double* inv_mass_type,
                         const double* mass_type, double* acc, double* v, double dt, double* th, double* ke,
                         cudaStream_t st);
void launch_md_berend(int nframes, const FramesDev& F, const double* mass_type, double* v, double dt, double tau,
                      double T0, double kb, double* ke, int* bad, cudaStream_t st);
// Conserved-quantity term per frame: mode 1 NVT-MTK, 2 NPT-MTK (with p0 V), 0 none.
void launch_md_conserved(int nframes, const double* th, int mode, double p0, const BoxDev* box, double* out,
                         cudaStream_t st);

}  // namespace cgd
