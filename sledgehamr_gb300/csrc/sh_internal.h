/* Internal types shared by the CUDA translation units of
 * libsledgehamr_gb300.so.  Nothing here is part of the C ABI
 * (include/sledgehamr_gb300.h).
 *
 * Device data layout of a level ("level buffer"): the boxes of the level one
 * after the other; inside a box every component is a contiguous FP64 array
 * over the ghost-grown box, x fastest, then y, z, component - the FArrayBox
 * layout of the reference, so that project hooks index it through the same
 * Array4 semantics.  Per-stage accumulator buffers ("K buffers") use the same
 * box layout with only the components the integrator keeps.
 */
#ifndef SH_INTERNAL_H_
#define SH_INTERNAL_H_

#include <cuda_runtime.h>

#include <cstdint>
#include <string>
#include <vector>

#include "sh_fill_plan.h" /* GhostCopyDev, CfRect, FillPlan */

struct sh_ctx;

namespace sh {

/* Replaces the context's last error message (sh_ctx_last_error); for the
 * library's host layers (the AMR hierarchy) that report their own errors
 * through a context. */
void set_ctx_error(::sh_ctx *ctx, const std::string &msg);

constexpr int kMaxParams = 32;   /* doubles of Rhs parameters per call */
constexpr int kMaxGwParams = 16; /* doubles of GW Rhs parameters per call */
constexpr int kMaxComp = 32;     /* components per level */
constexpr int kMaxStages = 8;    /* RKN stages */

/* Tile of a box processed by one thread block of the stage kernels. */
/* Stage tiles: up to kTileX cells in x, kThreads / nx rows in y and
 * kTileZ planes in z (kTileZShallow on levels whose deep tiles would not
 * fill two waves of the GPU). */
constexpr int kTileX = 32, kTileY = 4, kTileZ = 32, kTileZShallow = 8;
constexpr int kThreads = kTileX * kTileY;

struct BoxDev {
    long long off;  /* element offset of the box in a level buffer (per comp-set) */
    long long gvol; /* cells of the ghost-grown box */
    int lo[3];      /* valid box */
    int hi[3];
    int glo[3];     /* ghost-grown lower corner */
    int gdim[3];    /* ghost-grown extents */
};

struct TileDev {
    int box;
    int x0, y0, z0; /* first cell of the tile (absolute level index) */
    int nx;         /* cells along x (<= kTileX); the tile has kThreads / nx rows */
    int nz;         /* planes along z */
};


/* Which epilogue follows the per-cell Rhs evaluation in a stage kernel. */
enum EpilogueKind : int {
    kEpiPlainRhs = 0, /* rhs_out = f(state), all components */
    kEpiRknStage = 1, /* K_i = accel; Y_{i+1} positions (+ momenta copy) */
    kEpiRknFinal = 2, /* y1 from y0 and all K_i */
    kEpiSsp0 = 3,     /* K = f; u = y0 + a K */
    kEpiSspAdd = 4,   /* K = f + w K_old; u = y0 + a K (write K if kout) */
    kEpiLf0 = 5,      /* vh = v0 + dt/2 a; x1 = x0 + dt vh */
    kEpiLf1 = 6,      /* v1 = vh + dt/2 a; positions copied */
    kEpiRknFinalNoKqPos = 7 /* kEpiRknFinal when the last bbar is zero */
};

/* Kernel argument block of a stage kernel (passed by value as a
 * __grid_constant__ parameter, so `params` can be handed to project hooks as
 * a device pointer without a host-to-device copy). */
struct StageArgs {
    const TileDev *tiles;
    const BoxDev *boxes;
    const double *state; /* stage state read by the hooks (with ghosts) */
    const double *y0;    /* state at the start of the step */
    double *out;         /* next stage state or result */
    double *kout;        /* K buffer written by this stage (or nullptr) */
    const double *kin[kMaxStages];
    int nkin;
    int epi;
    int lev;
    int ncomp;   /* components of the level */
    int nk;      /* components in K buffers */
    int npair;   /* position/momentum pairs (user + GW) */
    int pos[kMaxComp / 2];
    int mom[kMaxComp / 2];
    double time, dt, dx;
    /* a level of one box covering its periodic domain (extent per[d], ng
     * ghost cells): the stage kernel also writes every output value into
     * the ghost cells that are periodic images of its cell, so that no
     * separate ghost fill is needed (0: ghost cells left to the fill; set
     * only without Kreiss-Oliger dissipation) */
    int self_periodic;
    int ng;
    int per[3];
    double c_mom;                /* coefficient of y0' in the stage positions */
    double c_k[kMaxStages];      /* coefficients of K_j in the stage positions */
    double c_k2[kMaxStages];     /* coefficients of K_j in the momenta (final) */
    double weight;               /* FillAddRhs weight */
    double c_out;                /* coefficient of K in u = y0 + c K */
    double params[kMaxParams];
    double gw_params[kMaxGwParams];
    double ko_strength[kMaxComp];
};

/* Launch description handed to a project's stage launcher. */
struct StageLaunch {
    StageArgs args;
    int ntiles;
    bool with_gw;
    int ko_order; /* 0, 2 or 3 */
};

struct TagArgs {
    const BoxDev *boxes;
    const TileDev *tiles;
    const double *state;
    const double *te; /* nullptr: no truncation-error tags */
    unsigned char *mask; /* per box valid cells, box-major (offsets in mask_off) */
    const long long *mask_off;
    unsigned long long *counts; /* [0] total, [1] user, [2+n] per component */
    int ncomp;
    int lev;
    double time, dt, dx;
    double te_crit[kMaxComp];
    double params_tag[kMaxParams];
    double params_mod[kMaxComp];
};

/* Entry points a project translation unit provides. */
struct ProjectOps {
    const char *name;
    int nscalars;  /* user fields including momenta */
    int nfields;   /* position fields */
    bool has_gw;   /* the project supplies GravitationalWavesRhs<true> */
    int reach;     /* largest neighbour offset its hooks read */
    const char *(*field_name)(int comp); /* user field names, NULL past them */
    cudaError_t (*launch_stage)(const StageLaunch &, cudaStream_t);
    cudaError_t (*launch_tag)(const TagArgs &, int ntiles, cudaStream_t);
};

const ProjectOps *project_by_id(int id);
int project_count();

/* Projects register themselves when the library loads (SH_DEFINE_PROJECT
 * makes one of these per project translation unit), so that adding a
 * project is adding its headers and one .cu file, without editing a list. */
void register_project(const ProjectOps *p);
struct ProjectRegistrar {
    explicit ProjectRegistrar(const ProjectOps *p) { register_project(p); }
};

} // namespace sh

#endif // SH_INTERNAL_H_
