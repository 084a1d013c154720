/* C ABI of libsledgehamr_gb300.so: sledgehamr's time-stepping hot path on one
 * GB300 GPU.
 *
 * The library replaces, for a host driver written in C, C++ or Python
 * (ctypes), the AMReX-backed operations that sledgehamr's TimeStepper calls on
 * every step:
 *   sh_level_advance ........ Integrator::Advance + IntegratorRkn/Lsssprk3/
 *                             Leapfrog::Integrate
 *                             (source/integrators/integrator.cpp:11-31,
 *                              rkn.cpp:25-120, lsssprk3.cpp:14-31,
 *                              leapfrog.cpp:13-57), including the project's
 *                             FillRhs/FillAddRhs (source/macros.h:301-485)
 *   sh_level_fill_patch ..... LevelSynchronizer::FillPatch for lev <= 0
 *                             (source/level_synchronizer.cpp:94-144)
 *   sh_level_rhs ............ Sledgehamr::FillRhs (macros.h:301-379)
 *   sh_average_down ......... LevelSynchronizer::AverageDownTo and the
 *                             average-down of CreateShadowLevel
 *                             (level_synchronizer.cpp:219-233,
 *                              sledgehamr.cpp:247-248)
 *   sh_average_down_te ...... LevelSynchronizer::ComputeTruncationErrors
 *                             (level_synchronizer.cpp:240-357, kernels.h:18-42)
 *   sh_tag .................. Sledgehamr::ErrorEst / DoErrorEstCpu
 *                             (sledgehamr.cpp:207-348, macros.h:489-686)
 *   sh_gw_spectrum .......... GravitationalWaves::ComputeSpectrum
 *                             (gravitational_waves.cpp:52-322)
 *   sh_spectrum_bins,
 *   sh_index_to_k ........... Sledgehamr::ReadSpectrumKs / ReadProj data
 *                             (sledgehamr.cpp:554-615, generated as
 *                              pySledgehamr/Sledgehamr.py:7-27)
 *   sh_level_reduce ......... LevelData::norm0 / MultiFab::sum of the
 *                             projects' host code
 *                             (FirstOrderPhaseTransition.cpp:133-157,
 *                              NextToMinimalExample.cpp:35)
 *   sh_h5_*, sh_output_* .... the HDF5 files of the output types: the
 *                             dataset writer utils::hdf5::Write
 *                             (source/utils/hdf5_utils.h:80-104),
 *                             LevelWriter::WriteSingleLevel
 *                             (output_types/level_writer.h:80-171) and
 *                             Slices::Write (output_types/slices.cpp:13-145)
 *   sh_amr_* ................ TimeStepper::Advance / Sledgehamr::Evolve over
 *                             a whole hierarchy (time_stepper.cpp:90-397)
 *   sh_evolve_periodic ...... host-to-host convenience: upload, nsteps x
 *                             Advance(0), download, for a periodic cubic level
 *
 * Projects (per-cell hooks) are compiled into the library; see
 * sh_project_find.  Component order of a level: the project's fields, then
 * its momenta (SLEDGEHAMR_ADD_SCALARS / ADD_CONJUGATE_MOMENTA), then, when
 * gravitational waves are on, u_xx u_yy u_zz u_xy u_xz u_yz du_xx ... du_yz.
 *
 * Host array layouts:
 *   canonical  - one array for a level covering its whole cubic periodic
 *                domain of N^3 cells: a[((n*N + k)*N + j)*N + i]
 *   boxes      - the valid cells of every box one after the other, each box
 *                component-major, x fastest.
 *
 * Every function returns SH_OK (0) or a negative status; the message of the
 * last failure is available from sh_ctx_last_error.  No function aborts the
 * process.  Calls on one context are not thread-safe; different contexts
 * are independent.  All work is issued on the context's stream; functions
 * that take or return host arrays synchronise that stream before returning.
 */
#ifndef SLEDGEHAMR_GB300_H_
#define SLEDGEHAMR_GB300_H_

#include <stddef.h>
#include <stdint.h>

#if defined(__GNUC__)
#define SH_API __attribute__((visibility("default")))
#else
#define SH_API
#endif

#ifdef __cplusplus
extern "C" {
#endif

#define SH_OK 0
#define SH_ERR_ARG (-1)
#define SH_ERR_PROJECT (-2)
#define SH_ERR_CUDA (-3)
#define SH_ERR_NOMEM (-4)
#define SH_ERR_UNSUPPORTED (-5)
#define SH_ERR_TIMEOUT (-6)
#define SH_ERR_NONFINITE (-7)

/* integrator.type (source/integrators/integrator.h:12-23).  The AMReX
 * integrators 0-4 abort in the reference (amrex_integrators.cpp:19-20) and
 * are rejected here with SH_ERR_UNSUPPORTED. */
#define SH_INTEGRATOR_LSSSPRK3 10
#define SH_INTEGRATOR_LEAPFROG 11
#define SH_INTEGRATOR_RKN_TABLEAU 20
#define SH_INTEGRATOR_RKN4 21
#define SH_INTEGRATOR_RKN5 22

/* sh_level_advance flags */
#define SH_ADVANCE_NO_SWAP 1 /* shadow level: integrate old -> new in place
                                of swapping first (integrator.cpp:12-15) */

/* which time level of a sh_level */
#define SH_NEW 0
#define SH_OLD 1

typedef struct sh_ctx sh_ctx;
typedef struct sh_level sh_level;

/* An index box, bounds inclusive, as amrex::Box. */
typedef struct sh_box {
    int lo[3];
    int hi[3];
} sh_box;

/* ---- context -------------------------------------------------------------- */
SH_API int sh_ctx_create(int device, sh_ctx **out);
SH_API int sh_ctx_destroy(sh_ctx *ctx);
SH_API const char *sh_ctx_last_error(const sh_ctx *ctx);
/* Use an existing cudaStream_t (NULL: the context's own stream). */
SH_API int sh_ctx_set_stream(sh_ctx *ctx, void *cuda_stream);
SH_API void *sh_ctx_stream(sh_ctx *ctx);
SH_API int sh_ctx_synchronize(sh_ctx *ctx);
/* Number of kernels this context has launched so far. */
SH_API long long sh_ctx_kernel_launches(const sh_ctx *ctx);
/* Per-kernel timing with CUDA events recorded on the context stream around
 * every launch while enabled (the categories of sledgehamr's
 * PerformanceMonitor: "rhs" (stage kernels), "fill_patch" (same-level
 * ghost copies and level-to-level copies), "coarse_fine" (ghost cells
 * interpolated from the coarse level), "average_down", "tagging",
 * "gw_spectrum", "data_move").  sh_ctx_profile(ctx, 1) clears
 * and starts, (ctx, 0) stops; sh_ctx_profile_read synchronises the stream
 * and returns the summed device time and the launch count of a category. */
SH_API int sh_ctx_profile(sh_ctx *ctx, int enable);
SH_API int sh_ctx_profile_read(sh_ctx *ctx, const char *category, double *total_ms,
                               long long *launches);

/* ---- projects ------------------------------------------------------------- */
SH_API int sh_project_count(void);
SH_API const char *sh_project_name(int id);
SH_API int sh_project_find(const char *name, int *id);
/* Components of a level of the project (with_gw adds the 12 tensor
 * components) and the number of field/momentum pairs. */
SH_API int sh_project_ncomp(int id, int with_gw, int *ncomp, int *npairs);
/* Name of component comp of a level of the project: the names given to
 * SLEDGEHAMR_ADD_SCALARS / ADD_CONJUGATE_MOMENTA, then u_xx ... du_yz
 * (Sledgehamr::GetScalarFieldName, source/sledgehamr.h:142-144).  The
 * string is owned by the library. */
SH_API int sh_project_comp_name(int id, int comp, const char **name);

/* ---- levels ---------------------------------------------------------------- */
/* A level of one project: boxes inside the periodic domain [dlo, dhi], with
 * nghost ghost cells, holding two time levels (SH_NEW, SH_OLD) as
 * sledgehamr's grid_new/grid_old, plus the scratch the integrators need. */
SH_API int sh_level_create(sh_ctx *ctx, int project, int with_gw, const int domain_lo[3],
                    const int domain_hi[3], const sh_box *boxes, int nbox, int nghost,
                    sh_level **out);
/* sh_level_create with a storage precision: SH_PREC_FP64 (the reference's
 * FArrayBox data), or SH_PREC_FP32_KAHAN, the precision form on levels:
 * FP32 values with FP32 Kahan compensations (value v and compensation c
 * stand for v - c), advanced by FP32 stage kernels written against the
 * equations (the axion-string projects AxionStringsLap1 / Lap2 with RKN4,
 * no GW tensor; FirstOrderPhaseTransition with the pure potential and the
 * leapfrog, with or without GW tensor), FP32 ghost fills and average-down
 * (sums as FP32 TwoSum pairs), while time, truncation errors (kept in
 * FP64), tagging through the project's hooks, reductions, spectra and
 * outputs work on the FP64 values v - c.  Reads, writes and bubble
 * injection convert; the Rhs hook (sh_level_rhs) and sh_tag_static need
 * FP64 levels (SH_ERR_UNSUPPORTED).  No reference counterpart (sledgehamr
 * stores FP64 only). */
SH_API int sh_level_create_prec(sh_ctx *ctx, int project, int with_gw,
                                const int domain_lo[3], const int domain_hi[3],
                                const sh_box *boxes, int nbox, int nghost, int precision,
                                sh_level **out);
SH_API int sh_level_precision(const sh_level *level, int *precision);
SH_API int sh_level_destroy(sh_ctx *ctx, sh_level *level);
/* Index domain of a level (lo, hi inclusive). */
SH_API int sh_level_domain(const sh_level *level, int lo[3], int hi[3]);
/* Project id of a level and whether it carries the tensor components. */
SH_API int sh_level_project(const sh_level *level, int *project, int *with_gw);
SH_API int sh_level_info(const sh_level *level, int *ncomp, int *nbox, long long *nvalid_cells);
SH_API int sh_level_time(const sh_level *level, int which, double *t, int *istep);
/* Box list of a level (capacity boxes; *nbox receives the count). */
SH_API int sh_level_boxes(const sh_level *level, sh_box *out, int capacity, int *nbox);
/* AMR level index handed to the project hooks as `lev` (default 0; the
 * shadow level is -1). */
SH_API int sh_level_set_index(sh_level *level, int lev);
SH_API int sh_level_set_time(sh_level *level, int which, double t, int istep);

/* Copy valid cells between host and a time level (layout 0: canonical,
 * which requires one cubic domain covered by the level's boxes; layout 1:
 * boxes).  Ghost cells are not touched. */
SH_API int sh_level_write(sh_ctx *ctx, sh_level *level, int which, int layout, const double *host);
SH_API int sh_level_read(sh_ctx *ctx, const sh_level *level, int which, int layout, double *host);
/* Same with device arrays, asynchronous on the context stream. */
SH_API int sh_level_write_device(sh_ctx *ctx, sh_level *level, int which, int layout,
                          const double *dev);
SH_API int sh_level_read_device(sh_ctx *ctx, const sh_level *level, int which, int layout,
                         double *dev);

/* Ghost cells of one time level from the valid cells of the same level,
 * periodic in every direction (FillPatch / FillIntermediatePatch for
 * lev <= 0). */
SH_API int sh_level_fill_patch(sh_ctx *ctx, sh_level *level, int which);

/* Link a fine level to its coarse level (NULL unlinks).  From then on the
 * fine level's FillPatch (sh_level_fill_patch, and the fills inside
 * sh_level_advance) fills the ghost cells not covered by the fine level's own
 * boxes by quadratic interpolation (amr.interpolation_type CellQuadratic)
 * from the coarse data at the fill time, linearly interpolated in time
 * between the coarse level's OLD and NEW time levels (LevelSynchronizer::
 * FillPatch / FillIntermediatePatch for lev > 0,
 * source/level_synchronizer.cpp:94-214, :613-632).  The coarse level must
 * cover the parents of those cells and have nghost >= 1 with filled ghosts;
 * the link must be renewed when either level's boxes change. */
SH_API int sh_level_set_coarse(sh_ctx *ctx, sh_level *fine, sh_level *coarse);
/* Fill time level which_dst of dst (valid and ghost cells) from the valid
 * cells of src (time level which_src; any box layout of the same domain,
 * may be NULL) and interpolate the cells src does not cover from `coarse` at
 * `time` (LevelSynchronizer::FillCoarsePatch when src is NULL,
 * level_synchronizer.cpp:56-82; RemakeLevel's FillPatch otherwise,
 * sledgehamr.cpp:173-189). */
SH_API int sh_level_fill_from(sh_ctx *ctx, sh_level *dst, int which_dst, const sh_level *src,
                              int which_src, sh_level *coarse, double time);

/* One step of integrator `integrator` (SH_INTEGRATOR_*) of a periodic
 * level: swap(new, old) unless SH_ADVANCE_NO_SWAP, FillPatch(old), integrate
 * old -> new, t_new = t_old + dt, istep_new = istep_old + 1.
 * tableau (type 20 only): nodes[s], bbar[s], b[s], then the lower triangle
 * of a including the diagonal, row by row.  params/gw_params: the vectors
 * that SetParamsRhs / SetParamsGravitationalWaveRhs produce (at most 32 and
 * 16 doubles).  ko_order 0 (off), 2 or 3 with ko_strength[ncomp].
 * Every stage's output, new included, leaves with its ghost cells filled
 * (FillIntermediatePatch); on an FP64 level of one box covering its periodic
 * domain without dissipation the stage kernels write those periodic images
 * themselves, with the same values. */
SH_API int sh_level_advance(sh_ctx *ctx, sh_level *level, int integrator, const double *tableau,
                     int nstages, double dt, double dx, const double *params, int nparams,
                     const double *gw_params, int ngw, int ko_order, const double *ko_strength,
                     int flags);

/* rhs = f(state) (FillRhs) for the valid cells of time level `which`
 * (ghosts must be filled); result in boxes layout on the host. */
SH_API int sh_level_rhs(sh_ctx *ctx, sh_level *level, int which, double time, int lev, double dt,
                 double dx, const double *params, int nparams, const double *gw_params,
                 int ngw, int ko_order, const double *ko_strength, double *host_rhs);

/* Output functions for projections and scalar spectra (the projects'
 * io_module->projections / ->spectra functions, evaluated on the device):
 * a component, its square (FirstOrderPhaseTransition dPhi2 with comp 1),
 * and the AxionStrings densities of kernels_energy_densities.h (components
 * Psi1 Psi2 Pi1 Pi2 at 0..3; a_prime2 is also NextToMinimalExample's
 * a_dot_sq). */
#define SH_OUT_COMPONENT 0
#define SH_OUT_COMPONENT_SQ 1
#define SH_OUT_A_PRIME2 2
#define SH_OUT_A_PRIME_SCREENED 3
#define SH_OUT_R_PRIME2 4

/* Spectrum::Compute (source/output_types/spectrum.cpp:12-113) of a level
 * covering its whole cubic periodic domain: the output function per cell,
 * its R2C FFT, and per bin of the sorted unique k^2 (as sh_spectrum_bins)
 * the sum of multpl |F|^2 times t / (N^6 dk), dk = 2 pi / (N dx), t the
 * level's SH_NEW time, multpl = 1 on the x planes 0 and N/2, else 2. */
SH_API int sh_scalar_spectrum(sh_ctx *ctx, const sh_level *level, int fn, int comp, double dx,
                              double *bins_out, long long *ks_out, int max_bins, int *nbins);
/* Projection::Compute / Add (source/output_types/projection.cpp:10-118):
 * line-of-sight projection along z of the output function over levels
 * 0..nlev-1 (SH_NEW data) onto the pixel grid of the finest one (dimN^2,
 * data_out[x dimN + y]); a cell of level l not covered by level l+1 covers
 * ratio^2 pixels (ratio = dimN / dimN_l); mode 0 sums ratio * value, mode 1
 * keeps the maximum (starting from 0); n_out counts the contributions.
 * Levels must cover periodic cubic domains starting at 0, each twice the
 * previous. */
SH_API int sh_projection(sh_ctx *ctx, const sh_level *const *levels, int nlev, int fn,
                         int comp, int mode, double *data_out, int *n_out);

/* FirstOrderPhaseTransition bubble injection (InjectBubbles ->
 * AddBubbleValues, projects/FirstOrderPhaseTransition/
 * FirstOrderPhaseTransition.cpp:308-328, 459-483; AddBubble,
 * kernels_misc.h:27-52): every valid cell (i, j, k) at position
 * (i dx, j dx, k dx) of the periodic cubic domain adds, for each of the nb
 * bubbles (centres xyz[3 b + d]) in order, the profile at its periodic
 * distance D, linearly interpolated in bins of width 1/inv_dx:
 * profile[ind] (1 - f) + profile[ind + 1] f with D inv_dx = ind + f, to
 * component comp_phi (profile row 0, nbins values) and comp_dphi (row 1);
 * cells with D >= Lcut are unchanged.  nbins >= floor(Lcut inv_dx) + 2. */
SH_API int sh_level_add_bubbles(sh_ctx *ctx, sh_level *L, int which, int comp_phi,
                                int comp_dphi, int nb, const double *xyz,
                                const double *profile, int nbins, double inv_dx, double Lcut,
                                double dx);

/* Reduction of component comp over the valid cells of a time level:
 * SH_REDUCE_MAX_ABS (AMReX MultiFab::norm0, which FirstOrderPhaseTransition
 * uses for its TruncationModifier parameters, FirstOrderPhaseTransition.cpp:
 * 133-157), SH_REDUCE_MIN, SH_REDUCE_MAX, SH_REDUCE_SUM, SH_REDUCE_SUM_SQ
 * (MultiFab::sum of the component or of its square).  Sums are formed in
 * FP64 in a fixed order (per box, then over the boxes in order), so a
 * result is reproducible bit for bit.  Synchronises the context's stream.
 * Replaces the norm0 / sum calls of the reference's host code
 * (FirstOrderPhaseTransition.cpp:147, NextToMinimalExample.cpp:35). */
#define SH_REDUCE_MAX_ABS 0
#define SH_REDUCE_MIN 1
#define SH_REDUCE_MAX 2
#define SH_REDUCE_SUM 3
#define SH_REDUCE_SUM_SQ 4
/* SH_REDUCE_COUNT_NONFINITE: the number of NaN or infinite values of comp
 * (no counterpart in the reference; see sh_level_check_finite).
 * SH_REDUCE_SUM_MODULUS: the sum over the cells of sqrt(comp^2 +
 * (comp+1)^2), the radial mode r = |Psi| of NextToMinimalExample::WriteAvg
 * (projects/NextToMinimalExample/NextToMinimalExample.cpp:10-49), whose
 * <r> is this sum over the number of cells. */
#define SH_REDUCE_COUNT_NONFINITE 5
#define SH_REDUCE_SUM_MODULUS 6
SH_API int sh_level_reduce(sh_ctx *ctx, const sh_level *level, int which, int op, int comp,
                           double *out);
/* Every component of a time level checked for NaN and infinite values on
 * the valid cells: SH_OK, or SH_ERR_NONFINITE with *nonfinite (may be NULL)
 * the number of such values and the first affected component named in
 * sh_ctx_last_error.  The reference has no such check (a non-finite field
 * runs on silently). */
SH_API int sh_level_check_finite(sh_ctx *ctx, const sh_level *level, int which,
                                 long long *nonfinite);
/* Cosmology::GetStringTags (projects/AxionStrings/cosmology.cpp:114-142):
 * the number of valid cells of time level NEW whose project
 * TagCellForRefinement<true> hook is true (for the axion projects: cells
 * whose plaquettes are pierced by a string) at the given time, level index,
 * dt and dx.  Ghost cells must be current (+1 neighbours are read). */
SH_API int sh_level_string_tags(sh_ctx *ctx, sh_level *level, double time, int lev, double dt,
                                double dx, const double *params_tag, int nparams_tag,
                                long long *ntags);
/* Cosmology::Xi (cosmology.cpp:89-108, cosmology.h:77-97): the string
 * length parameter xi from a string-tag count on a level of spacing dx in a
 * box of comoving size L at conformal time eta (T1 = 5.4954174414835757e17,
 * m_pl = 1.22e19, g_* = 106).  Host arithmetic only. */
SH_API int sh_string_xi(long long string_tags, double dx, double L, double eta, double *xi);

/* ---- level synchronisation ------------------------------------------------- */
/* crse(which_c) = 2x2x2 average of fine(which_f) on every coarse cell
 * covered by a fine box. */
SH_API int sh_average_down(sh_ctx *ctx, const sh_level *fine, int which_f, sh_level *crse,
                    int which_c);
/* Truncation errors: for every coarse cell covered by fine(NEW),
 * te = |crse(NEW) - avg(fine)| is stored in fine(OLD) at the even fine cell
 * (2i, 2j, 2k), and crse(NEW) = avg(fine). */
SH_API int sh_average_down_te(sh_ctx *ctx, sh_level *fine, sh_level *crse);

/* ---- tagging ---------------------------------------------------------------- */
/* Tags of time level NEW (ghosts must be filled) with the project's
 * TagCellForRefinement<true>; if use_te, also the truncation errors stored
 * in time level OLD, modified by TruncationModifier<n> and compared with
 * te_crit[n].  mask_out (host, boxes layout, one byte per valid cell) gets 1
 * for tagged cells; counts_out (may be NULL) gets total, user and ncomp
 * per-component counts as sledgehamr's CPU tagger reports them;
 * list_out (may be NULL, room for list_capacity entries) gets the indices of
 * tagged cells in boxes layout, ascending, and *ntagged their number. */
SH_API int sh_tag(sh_ctx *ctx, sh_level *level, int use_te, double time, int lev, double dt,
           double dx, const double *te_crit, const double *params_tag, int nparams_tag,
           const double *params_mod, int nparams_mod, uint8_t *mask_out,
           long long *counts_out, int32_t *list_out, long long list_capacity,
           long long *ntagged);

/* Tagging for a regrid without the mask on the host: the tags of sh_tag
 * (same arguments), each tagged cell grown by `buffer` cells
 * (amr.n_error_buf) and coarsened to blocks of `block` cells of this level,
 * periodically wrapped: blocks_out[(bz * nb + by) * nb + bx] = 1 for every
 * block such a neighbourhood touches, nb = domain cells / block (cubic
 * domain).  ntagged = tagged cells (the CPU statistic of sh_tag).  Replaces
 * the host-side scan of the TagBoxArray that precedes clustering in
 * AmrCore::regrid / Sledgehamr::ErrorEst (sledgehamr.cpp:207-229). */
SH_API int sh_tag_blocks(sh_ctx *ctx, sh_level *level, int use_te, double time, int lev,
                         double dt, double dx, const double *te_crit, const double *params_tag,
                         int nparams_tag, const double *params_mod, int nparams_mod, int block,
                         int buffer, uint8_t *blocks_out, long long *ntagged);

/* Same tagging as sh_tag, for callers that must not allocate GPU memory:
 * hosts that hand out all device memory through their own pool or
 * allocator, or that cannot afford the device-wide synchronisation a
 * cudaMalloc/cudaFree implies in the middle of a step.  This entry point has
 * no counterpart in sledgehamr.  Its working memory (mask, tag list,
 * counters) is one fixed array inside the library, reserved on every GPU
 * that loads the library until the process exits; a level may hold at most
 * SH_TAG_STATIC_MAX_CELLS valid cells (larger levels get SH_ERR_ARG).  The
 * first call on a device looks up that array's device address, so make that
 * first call before capturing the stream into a CUDA graph.  All calls share
 * the array: calls whose GPU work overlaps (different streams or contexts on
 * one device) race and must be serialised by the caller. */
#define SH_TAG_STATIC_MAX_CELLS (1 << 22)
SH_API int sh_tag_static(sh_ctx *ctx, sh_level *level, int use_te, double time, int lev,
                         double dt, double dx, const double *te_crit,
                         const double *params_tag, int nparams_tag, const double *params_mod,
                         int nparams_mod, uint8_t *mask_out, long long *counts_out,
                         int32_t *list_out, long long list_capacity, long long *ntagged);

/* ---- gravitational-wave spectrum -------------------------------------------- */
/* Bins of unique k^2 (unbinned) for a dim^3 grid: sorted i^2+j^2+k^2 over the
 * integer FFT frequencies. */
SH_API int sh_spectrum_bins(int dim, long long *out, int capacity, int *nbins);
/* Effective momentum per index (projection_type 1: sin, 2: 4th-order, 3:
 * 6th-order central difference eigenvalue). */
SH_API int sh_index_to_k(int dim, int projection_type, double *out);
/* TT-projected GW spectrum of time level NEW of a level covering its cubic
 * domain with one box.  comps: the six tensor components (absolute component
 * indices, order xx xy xz yy yz zz); default (NULL): du_xx du_xy du_xz du_yy
 * du_yz du_zz.  Results in bins_out (capacity max_bins), number of bins in
 * *nbins and their k^2 in ks_out (may be NULL). */
SH_API int sh_gw_spectrum(sh_ctx *ctx, const sh_level *level, const int *comps, int zero_padding,
                   int projection_type, int unbinned, double *bins_out, long long *ks_out,
                   int max_bins, int *nbins);

/* ---- output files ------------------------------------------------------------ */
/* An HDF5 file of one-dimensional datasets in the root group, as sledgehamr's
 * utils::hdf5::Write creates them (source/utils/hdf5_utils.h:80-104): IEEE
 * little-endian F32 or F64 data, integers stored as F64.  Datasets are
 * collected by sh_h5_add and the file is written by sh_h5_write in the HDF5
 * library's default (earliest) file format; no HDF5 library is needed.
 * Names are unique, non-empty and without '/'.  Errors of the sh_h5_* and
 * sh_output_* calls are reported by sh_h5_last_error.  One sh_h5file is
 * used by one thread at a time; separate files are independent. */
typedef struct sh_h5file sh_h5file;
#define SH_H5_F32 4   /* float data, stored as F32LE */
#define SH_H5_F64 8   /* double data, stored as F64LE */
#define SH_H5_I32 -4  /* int32 data, stored as F64LE */
#define SH_H5_I64 -8  /* int64 data, stored as F64LE */
SH_API int sh_h5_create(sh_h5file **out);
SH_API int sh_h5_destroy(sh_h5file *f);
SH_API const char *sh_h5_last_error(const sh_h5file *f);
SH_API int sh_h5_add(sh_h5file *f, const char *name, int type, const void *data, long long n);
SH_API int sh_h5_count(const sh_h5file *f, long long *n);
SH_API int sh_h5_write(sh_h5file *f, const char *path);

/* The datasets of a level file (LevelWriter::WriteSingleLevel,
 * source/output_types/level_writer.h:80-171) added to f: time level NEW
 * under ident "data", or with truncation_error the truncation errors that
 * sh_average_down_te left in time level OLD under ident "te" (even cells
 * only, maximum per output cell).  Per box b (from 1) and component a
 * dataset "<name>_<ident>_<b>" of the box's cells, x slowest, averaged over
 * blocks of downsample^3 cells (a power of 2 dividing every box extent) in
 * precision 32 or 64; then Header_<ident> = {t, 1, finest_level, N,
 * downsample, boxes} and the box bounds lex_ ley_ lez_ hex_ hey_ hez_
 * (upper bounds exclusive).  sledgehamr writes one such file per level as
 * <folder>/Level_<lev>/0.hdf5. */
SH_API int sh_output_level(sh_ctx *ctx, const sh_level *level, int truncation_error,
                           int finest_level, int downsample, int precision, sh_h5file *f);
/* The three slices of a level file (Slices::Write,
 * source/output_types/slices.cpp:13-145): planes at index
 * floor(N * location[d]) (made even) normal to x, y and z, idents "x", "y",
 * "z" (or "te_x", "te_y", "te_z" for truncation errors), 32-bit floats per
 * box cutting the plane, Header_<ident> = {t, 1, finest_level, N, boxes}
 * and the bounds le1_ le2_ he1_ he2_. */
SH_API int sh_output_slices(sh_ctx *ctx, const sh_level *level, int truncation_error,
                            int finest_level, const double location[3], sh_h5file *f);
/* The same from host data: boxes and their valid cells in the boxes layout,
 * ncomp component names, the time and N of the level. */
SH_API int sh_output_level_host(const sh_box *boxes, int nbox, int ncomp, const double *cells,
                                const char *const *names, double t, int finest_level,
                                int dim_n, int truncation_error, int downsample, int precision,
                                sh_h5file *f);
SH_API int sh_output_slices_host(const sh_box *boxes, int nbox, int ncomp, const double *cells,
                                 const char *const *names, double t, int finest_level,
                                 int dim_n, int truncation_error, const double location[3],
                                 sh_h5file *f);

/* ---- AMR time stepping ---------------------------------------------------- */
/* A hierarchy of levels advanced with sledgehamr's recursive subcycling
 * (TimeStepper::Advance, source/time_stepper.cpp:90-171): each level takes
 * two steps per step of the level below, levels are averaged down after
 * their finer levels, and, when any te_crit is finite, regrids are scheduled
 * ahead of time with a shadow level (half resolution, twice the time step)
 * so that truncation errors are available at regrid time
 * (time_stepper.cpp:221-295, sledgehamr.cpp:234-251).  Tags combine the
 * project's TagCellForRefinement<true> with truncation errors (sh_tag);
 * new grids are blocking-factor blocks of the buffered tags merged into
 * boxes of at most max_grid_size cells. */
typedef struct sh_amr sh_amr;
typedef struct sh_amr_config {
    int project;                 /* sh_project_find id */
    int with_gw;
    int integrator;              /* integrator.type */
    int nghost;                  /* amr.nghost */
    int N0;                      /* amr.coarse_level_grid_size */
    int max_level;               /* amr.max_refinement_levels */
    int blocking_factor;         /* amr.blocking_factor */
    int max_grid_size;           /* grid size of every level */
    int n_error_buf;             /* amr.n_error_buf */
    int record_regrids;          /* keep tags and boxes of every regrid */
    double L;                    /* sim.L */
    double cfl;                  /* sim.cfl */
    double t_start;              /* sim.t_start */
    double regrid_dt;            /* amr.regrid_dt */
    double string_width_threshold; /* AxionStrings CreateLevelIf (<= 0: off) */
    double string_lambda;        /* lambda of the string width */
    double te_crit[32];          /* amr.te_crit per component (>= DBL_MAX: off) */
    double params[32];           /* SetParamsRhs */
    int nparams;
    double gw_params[16];        /* SetParamsGravitationalWaveRhs */
    int ngw;
    int clustering;              /* SH_CLUSTER_BR, SH_CLUSTER_WINDOWS, SH_CLUSTER_BR_WINDOWS */
    double grid_eff;             /* amr.grid_eff of the clustering (default 0.7) */
    double params_tag[32];       /* SetParamsTagCellForRefinement */
    int nparams_tag;
    double params_mod[32];       /* SetParamsTruncationModifier */
    int nparams_mod;
    /* 1: before the tagging of each regrid, params_mod[c] = max |comp c|
     * over the valid cells of level 0 (new time level), for every
     * component, as FirstOrderPhaseTransition's SetParamsTruncationModifier
     * does with norm0 (FirstOrderPhaseTransition.cpp:133-157); 0: params_mod
     * as given */
    int params_mod_norm0;
    /* 1: after every coarse step, every level's new time level is checked
     * for NaN and infinite values (sh_level_check_finite); sh_amr_step then
     * stops with SH_ERR_NONFINITE naming the level and component.  No
     * counterpart in the reference. */
    int check_finite;
    /* LocalRegrid (source/local_regrid/local_regrid.cpp): before a global
     * regrid, levels first grow by blocking-factor blocks next to their
     * coarse/fine boundaries where tagged cells come closer than
     * n_error_buf + 1 fine cells (lower levels growing to keep them
     * nested), keeping every existing box; at most max_local_regrids times
     * between global regrids (amr.max_local_regrids, 0: global regrids
     * only), vetoed in favour of a global regrid when a level would exceed
     * volume_threshold_weak times its volume at the last global regrid
     * (amr.volume_threshold_weak; volume_threshold_strong picks the level
     * to regrid globally). */
    int max_local_regrids;
    double volume_threshold_strong;
    double volume_threshold_weak;
    /* storage of every level: SH_PREC_FP64 (default) or SH_PREC_FP32_KAHAN
     * (sh_level_create_prec: AxionStringsLap1 / Lap2 with RKN4,
     * FirstOrderPhaseTransition with the leapfrog): the precision form on
     * hierarchies, with the truncation errors, tags and time in FP64 */
    int precision;
} sh_amr_config;
/* New-grid generation from the buffered tags (at blocking-factor
 * resolution): Berger-Rigoutsos clustering to efficiency grid_eff, then
 * chopping to max_grid_size, as AMReX's MakeNewGrids does (SH_CLUSTER_BR);
 * the same clustering run independently inside every aligned window of
 * max_grid_size cells, in parallel on the host (SH_CLUSTER_BR_WINDOWS); or
 * tagged blocks merged inside those windows, every box fully tagged
 * (SH_CLUSTER_WINDOWS). */
#define SH_CLUSTER_BR 0
#define SH_CLUSTER_WINDOWS 1
#define SH_CLUSTER_BR_WINDOWS 2

SH_API int sh_amr_config_defaults(sh_amr_config *cfg);
/* Hierarchy with level 0 = level0 (canonical layout, N0^3 cells, boxes of
 * max_grid_size) at t_start; level0 = NULL starts from a zero state (for
 * example to add bubbles to level 0 through sh_amr_level before the first
 * step). */
SH_API int sh_amr_create(sh_ctx *ctx, const sh_amr_config *cfg, const double *level0,
                         sh_amr **out);
SH_API int sh_amr_destroy(sh_ctx *ctx, sh_amr *amr);
/* n coarse steps (Sledgehamr::Evolve loop bodies). */
SH_API int sh_amr_step(sh_ctx *ctx, sh_amr *amr, int n);
/* New tagging parameters from the next regrid on (projects whose hooks
 * change them between steps, e.g. FirstOrderPhaseTransition's field maxima
 * for its TruncationModifier, FirstOrderPhaseTransition.cpp:133-157). */
SH_API int sh_amr_set_tag_params(sh_amr *amr, const double *params_tag, int nparams_tag,
                                 const double *params_mod, int nparams_mod);
SH_API int sh_amr_info(const sh_amr *amr, int *finest, long long *cell_updates, int *nregrids);
/* Host wall-clock seconds and call counts of the time stepper's phases
 * (q = 0, 1, ... until SH_ERR_ARG): advance, synchronize, shadow,
 * regrid.tag, regrid.new_grids, regrid.create, regrid.fill, regrid.destroy,
 * regrid.refresh.  With timer sync on, the device is waited for around every
 * timed phase (slower; for profiling).  The reference's PerformanceMonitor
 * (source/performance_monitor.h) keeps the same kind of per-phase timers. */
SH_API int sh_amr_set_timer_sync(sh_amr *a, int on);
SH_API int sh_amr_timer(const sh_amr *a, int q, const char **name, double *seconds,
                        long long *calls);
/* Level lev of the hierarchy (owned by it; valid until the next step). */
/* Operation trace of the time stepper (TimeStepper::Advance,
 * SynchronizeLevels, ScheduleRegrid, DoRegrid, CreateShadowLevel;
 * source/time_stepper.cpp:90-397, sledgehamr.cpp:234-251): with tracing on,
 * every operation appends one line "<op> <level> <time>" (op one of advance,
 * schedule, shadow, average_down, truncation_errors, regrid; times printed
 * exactly).  sh_amr_trace copies the lines so far (NUL-terminated) into buf
 * of cap bytes and stores their length; buf NULL: length only. */
/* Checkpoint::Write / Checkpoint::Read (source/output_types/checkpoint.cpp:
 * 18-187): the hierarchy's state between coarse steps to a folder (created
 * if missing): Meta.hdf5 with the reference's header datasets (Header,
 * blocking_factors, isteps, next_id, last_time_written) and this library's
 * (boxes, times, regrid schedule), and both time levels of every level as
 * raw FP64 files (the reference writes AMReX VisMF files there).
 * sh_amr_restart creates a hierarchy from such a folder with a
 * configuration describing the same grid; stepping it continues exactly as
 * the checkpointed hierarchy would have. */
SH_API int sh_amr_checkpoint(sh_ctx *ctx, sh_amr *amr, const char *folder);
SH_API int sh_amr_restart(sh_ctx *ctx, const sh_amr_config *cfg, const char *folder,
                          sh_amr **out);
SH_API int sh_amr_set_trace(sh_amr *amr, int on);
SH_API int sh_amr_trace(const sh_amr *amr, char *buf, long long cap, long long *len);
SH_API int sh_amr_level(const sh_amr *amr, int lev, sh_level **level);
/* Regrid record q (with record_regrids): the tagged level and time, its
 * boxes, its tag mask (boxes layout) and the new boxes of the level above. */
SH_API int sh_amr_regrid_record(const sh_amr *amr, int q, int *lev, double *time,
                                sh_box *tagged_boxes, int cap_tagged, int *n_tagged,
                                uint8_t *mask, long long cap_mask, long long *n_mask,
                                sh_box *new_boxes, int cap_new, int *n_new);

/* ---- diagnostics ---------------------------------------------------------------- */
/* Measured issue rate of FP64 fused multiply-adds on `device` (thread
 * instructions per second, all SMs, dependent chains with enough warps to
 * hide their latency): the peak of the FP64 roofline of the stage kernels.
 * No counterpart in the reference. */
SH_API int sh_probe_fp64_fma_rate(int device, double *fma_per_s);
/* The bounded wait of the tensor-copy stage kernels run on an mbarrier that
 * nothing completes, with a 2 ms limit: *status is SH_ERR_TIMEOUT when the
 * limit ended the wait (and the device stays usable).  No counterpart in
 * the reference. */
SH_API int sh_probe_wait_timeout(int device, int *status);

/* ---- convenience --------------------------------------------------------------- */
/* Evolve a periodic cubic level of N^3 cells (boxes of max_grid cells per
 * side, max_grid <= 0: one box) by nsteps steps; host arrays in canonical
 * layout.  init_new (may be NULL): content of the second time level before
 * the first step. */
SH_API int sh_evolve_periodic(sh_ctx *ctx, int project, int integrator, const double *tableau,
                       int nstages, int N, int max_grid, int nghost, int ncomp, int with_gw,
                       const double *state_in, const double *init_new, double *state_out,
                       double t0, double dt, double dx, int nsteps, const double *params,
                       int nparams, const double *gw_params, int ngw, int ko_order,
                       const double *ko_strength);

/* ------------------------------------------------------------------------ */
/* Ensembles: many periodic cubes (realisations) of one physics family,
 * stepped together by one set of fused stage-kernel launches per step, in
 * FP64 or in FP32 with Kahan-compensated state updates.  No counterpart in
 * the reference, which evolves one simulation per process; the equations
 * and integrators are those of the projects named below.
 *
 *   SH_FAMILY_AXION_LAP1/2  Psi1 Psi2 Pi1 Pi2 (ncomp 4), RKN4
 *       Pi' = -2 Pi/t + lap Psi - lambda Psi [t^2 (|Psi|^2 - 1) + c]
 *       (AxionStringsLap1/2 of this library; 7- / 13-point Laplacian);
 *       params per realisation: {lambda, c, 0, 0}.
 *   SH_FAMILY_FOPT_GW       Phi dPhi u_xx u_yy u_zz u_xy u_xz u_yz du_xx ..
 *       du_yz (ncomp 14, the level order), leapfrog (kick-drift-kick),
 *       4th-order stencils (FirstOrderPhaseTransition with GW, pure potential);
 *       params per realisation: {q2, q3, q4, 0}.
 *
 * Host arrays of one realisation are canonical (component-major, N^3 cells,
 * x fastest).  Realisation r has N[r]^3 cells and spacing dx[r]. */
#define SH_FAMILY_AXION_LAP1 1
#define SH_FAMILY_AXION_LAP2 2
#define SH_FAMILY_FOPT_GW 3
#define SH_PREC_FP64 0
#define SH_PREC_FP32_KAHAN 1
#define SH_PREC_FP32 2

typedef struct sh_ensemble sh_ensemble;

SH_API int sh_ensemble_create(sh_ctx *ctx, int family, int precision, int nreal, const int *N,
                              const double *dx, const double *params, sh_ensemble **out);
SH_API int sh_ensemble_destroy(sh_ensemble *e);
SH_API const char *sh_ensemble_last_error(const sh_ensemble *e);
SH_API int sh_ensemble_info(const sh_ensemble *e, int *family, int *precision, int *nreal,
                            int *ncomp, long long *cells, long long *device_bytes, int *tile_nz);
SH_API long long sh_ensemble_kernel_launches(const sh_ensemble *e);
/* Time of the state (all realisations share it). */
SH_API int sh_ensemble_set_time(sh_ensemble *e, double t);
SH_API int sh_ensemble_time(sh_ensemble *e, double *t);
/* Upload / download realisation r (FP64 host values; an upload clears the
 * compensation, a download returns value minus compensation). */
SH_API int sh_ensemble_write(sh_ensemble *e, int r, const double *host);
SH_API int sh_ensemble_read(sh_ensemble *e, int r, double *host);
/* nsteps steps of size dt; asynchronous on the context's stream.  With
 * graphs on, every step replays a CUDA graph of its kernels. */
SH_API int sh_ensemble_set_graph(sh_ensemble *e, int on);
SH_API int sh_ensemble_step(sh_ensemble *e, double dt, int nsteps);
/* Tile depth along z; 0 times {4, 8, 16, 32, 64} on the current state
 * (leaving state, compensation and time unchanged) and keeps the fastest,
 * for each stencil-plane staging the ensemble allows (see below). */
SH_API int sh_ensemble_tune(sh_ensemble *e, int tile_nz, double dt, int *chosen);
/* Stencil-plane staging of the axion stage kernels: 0 planes loaded through
 * registers into a shared-memory ring; 1 planes brought into shared memory
 * by the Tensor Memory Accelerator (tiled tensor copies, two planes in
 * flight; FP32 storage, every realisation's N a multiple of 4 and at most
 * 256, else SH_ERR_UNSUPPORTED).  Both give the same results.  A stage
 * kernel whose wait for its copies runs out (one second) records
 * SH_ERR_TIMEOUT, which the next synchronising call of the ensemble
 * returns. */
SH_API int sh_ensemble_set_staging(sh_ensemble *e, int staging);
SH_API int sh_ensemble_staging(const sh_ensemble *e, int *staging);
/* Diagnostics per realisation: total energy (FP64 sums of the densities
 * listed at energy_kernel), number of string-pierced cells (axion
 * families; plaquette winding as in AxionStrings tagging), GW spectrum of
 * realisation r (FOPT_GW; arguments as sh_gw_spectrum). */
SH_API int sh_ensemble_energy(sh_ensemble *e, double *energy);
SH_API int sh_ensemble_string_count(sh_ensemble *e, long long *counts);
/* Pools: an ensemble with room for capacity_cells cells per array
 * (0: 80% of the free device memory) whose members are admitted and
 * released one by one; a member has its own N, dx, params and step dt
 * (FOPT_GW; sh_ensemble_step with dt = 0 advances every member by its own
 * dt).  Admission fails with SH_ERR_NOMEM while no free extent holds N^3
 * cells.  Slot numbers of released members are reused. */
SH_API int sh_ensemble_create_pool(sh_ctx *ctx, int family, int precision,
                                   long long capacity_cells, sh_ensemble **out);
SH_API int sh_ensemble_admit(sh_ensemble *e, int N, double dx, const double *params, double dt,
                             int *slot);
SH_API int sh_ensemble_release(sh_ensemble *e, int slot);
SH_API int sh_ensemble_pool_info(const sh_ensemble *e, long long *capacity,
                                 long long *free_cells, long long *largest_free, int *members);
/* Bubble injection into realisation r of an FOPT_GW ensemble, as
 * sh_level_add_bubbles (realisation side L = N dx). */
SH_API int sh_ensemble_add_bubbles(sh_ensemble *e, int r, int nb, const double *xyz,
                                   const double *profile, int nbins, double inv_dx,
                                   double Lcut);
SH_API int sh_ensemble_gw_spectrum(sh_ensemble *e, int r, int zero_padding, int projection_type,
                                   int unbinned, double *bins_out, long long *ks_out,
                                   int max_bins, int *nbins);
/* Precision of the GW spectrum's transforms and TT projection for this
 * ensemble: SH_PREC_FP64 (default; the FP64 drop-in's arithmetic) or
 * SH_PREC_FP32 (FP32 transforms and projection of the FP32 state, FP64
 * bin sums: the precision form's time-to-spectrum; its error against the
 * FP64 transform is stated by the benchmark).  No reference counterpart. */
SH_API int sh_ensemble_set_spectrum_precision(sh_ensemble *e, int precision);

/* ------------------------------------------------------------------------ */
/* Serving: a request loop over one FP32+Kahan (or FP64) pool of
 * FirstOrderPhaseTransition + GW runs (no counterpart in the reference).
 * A request is a periodic N^3 run from a zero state with bubbles injected
 * at t = 0 (as sh_level_add_bubbles), stepped by the leapfrog with step dt
 * until t_end, then its GW spectrum (as sh_gw_spectrum).  sh_server_step
 * admits queued requests while device memory is free (a request that does
 * not fit lets later ones pass until the oldest has waited 64 iterations),
 * advances all admitted runs by one step in shared launches, and finishes
 * the runs that reached t_end.  A request with max_level >= 1 runs instead
 * as its own AMR hierarchy (sh_amr: FP32 + Kahan levels on an FP32 server,
 * FP64 levels on an FP64 one; leapfrog with subcycling,
 * refinement by the truncation errors of Phi and dPhi against te_crit with
 * the TruncationModifier maxima of level 0, params_mod_norm0), admitted
 * while the device has room for 16 times its level-0 state and advanced to
 * t_end in a context (CUDA stream) and host thread of its own, so that its
 * kernels overlap with the pool's; its spectrum is taken from level 0 (the
 * fine levels averaged down) and collected by the next sh_server_step.
 * sh_server_destroy stops running hierarchies after their current step.
 * Times (seconds since the server's creation, host clock): submitted,
 * admitted, spectrum ready. */
typedef struct sh_request {
    int N;
    double dx, dt, t_end;
    double params[4];     /* q2 q3 q4 0 */
    int nbubbles;
    const double *xyz;    /* 3 per bubble (copied at submission) */
    const double *profile; /* 2 x nbins (copied) */
    int nbins;
    double inv_dx, Lcut;
    int zero_padding, projection_type, unbinned;
    int max_level;        /* 0: single level in the pool; 1, 2: AMR hierarchy */
    int blocking_factor;  /* AMR requests: amr.blocking_factor (0: 8) */
    int max_grid_size;    /* AMR requests: amr.max_grid_size (0: 32) */
    double te_crit[2];    /* AMR requests: te_crit of Phi and dPhi */
    double regrid_dt;     /* AMR requests: amr.regrid_dt */
} sh_request;
typedef struct sh_server sh_server;
SH_API int sh_server_create(sh_ctx *ctx, int precision, long long capacity_cells,
                            sh_server **out);
SH_API int sh_server_destroy(sh_server *s);
SH_API const char *sh_server_last_error(const sh_server *s);
SH_API int sh_server_submit(sh_server *s, const sh_request *r, long long *id);
SH_API int sh_server_step(sh_server *s, int *running, int *queued, int *completed);
/* state: 0 queued, 1 running, 2 done, 3 failed; times[3] as above. */
SH_API int sh_server_status(const sh_server *s, long long id, int *state, double *times);
SH_API int sh_server_result(const sh_server *s, long long id, double *bins, long long *ks,
                            int cap, int *nbins);
SH_API int sh_server_info(const sh_server *s, int *running, int *queued,
                          long long *cell_updates, long long *iterations,
                          long long *free_cells);

#ifdef __cplusplus
}
#endif

#endif /* SLEDGEHAMR_GB300_H_ */
