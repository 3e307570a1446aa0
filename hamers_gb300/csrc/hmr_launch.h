// Host-side launch interface between the C ABI (hmr_abi.cu) and the kernel
// translation units.  hmr_faces.cu is compiled twice: once in the exact form
// (namespace hmr_exact, --fmad=false) and once in the fast form (namespace
// hmr_fast).  hmr_cells.cu (cell data, sensor, ghost fill, elementwise RK
// stage) is always exact so both forms see identical sensor inputs.
#pragma once

#include <cuda_runtime.h>

#include "hmr_kernels.cuh"

namespace hmr {

struct Variant {
    int dim;
    int model;
    int nsp;
    int scheme;
};

// One entry of the batched worklist: a patch with its stage states.
struct PatchWork {
    Geom g;
    Scratch S;
    Comp Q[3];        // stage states (ghost box)
    Comp Qout;        // output of the substep
    int periodic[3];  // ghost fill of a patch that spans the domain: periodic axes (else zero-gradient)
    long off_fill;    // prefix offsets of the item counts, per phase
    long off_cells;
    long off_sensor;
    long off_face[3];
    long off_update;
};

struct LevelArgs {
    const PatchWork* work;   // device array
    int npatch;
    int ncomp;
    long total_fill, total_cells, total_sensor, total_face[3], total_update;
    double alpha[3];
    int nst;
    double beta;
    double dt;
    unsigned int* barrier;   // device counter for the grid barrier (zeroed before launch)
    int* status;             // device error flag (barrier give-up)
    unsigned long long timeout_ns;   // bound of every barrier wait
    unsigned int barrier_extra;      // diagnostic: arrivals that never come (0 in normal use)
    Redo redo;                       // faces handed from the fast to the exact form (count zeroed per launch)
};

}  // namespace hmr

namespace hmr_cells {
int launch_cells(const hmr::Variant& v, const hmr::Params& P, const hmr::Geom& g, const hmr::Comp& Q,
                 const hmr::Scratch& S, cudaStream_t st);
int launch_sensor(const hmr::Variant& v, const hmr::Geom& g, const hmr::Scratch& S, cudaStream_t st);
int launch_fill(int dim, const hmr::Geom& g, const hmr::Comp& Q, int ncomp, const int* periodic, cudaStream_t st);
int launch_rk_stage(const hmr::Variant& v, const hmr::Geom& g, int ncoef, const double* alpha,
                    const double* beta, const double* gamma, const hmr::Comp* Qint, const hmr::FluxComp* Fint,
                    const hmr::Comp* Sint, const hmr::Comp& Qout, const hmr::FluxComp& Facc, const hmr::Comp& Sacc,
                    cudaStream_t st);
}

#define HMR_DECLARE_FACE_LAUNCHERS(NS)                                                                       \
    namespace NS {                                                                                           \
    int launch_faces(const hmr::Variant& v, const hmr::Params& P, const hmr::Geom& g, const hmr::Scratch& S, \
                     hmr::Counters* cnt, const hmr::Redo& R, cudaStream_t st);                               \
    int launch_update(const hmr::Variant& v, const hmr::Geom& g, const hmr::Scratch& S,                      \
                      const hmr::UpdateArgs& U, cudaStream_t st);                                            \
    int launch_level(const hmr::Variant& v, const hmr::Params& P, const hmr::LevelArgs& L, int blocks,       \
                     int threads, cudaStream_t st);                                                          \
    int level_max_blocks(const hmr::Variant& v, int threads, int* blocks);                                   \
    }

HMR_DECLARE_FACE_LAUNCHERS(hmr_exact)
HMR_DECLARE_FACE_LAUNCHERS(hmr_fast)
