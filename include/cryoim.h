/*
 * cryoim.h — C ABI of libcryoim_gb300.so, the GB300 (sm_103a) implementation of
 * cryoIM's icosahedral projection-matching refinement loop.
 *
 * The reference (chenwenyuan2009/cryoIM) is Fortran 90 with all state in module
 * globals (icosprocess/SRC/0common_icosproc.f90:2-115) and no library API.  Every
 * entry point below replaces one Fortran subroutine (or driver loop) of that path
 * and is callable from Fortran through ISO_C_BINDING: plain pointers, int32/float
 * by value, no C++ or torch types, every function returns an int status
 * (CRYOIM_OK = 0, negative = error; nothing calls exit()).
 *
 * Ownership: the caller owns every host array.  Device memory lives inside an
 * opaque cryoim_ctx (one per host thread; a context is not thread safe).  Calls are
 * synchronous at the API edge unless the name ends in _async.  Entry points whose
 * name ends in _device take device pointers (resident in HBM) for their bulk
 * inputs; all others take host pointers and do the host<->device copies.
 *
 * Array conventions follow the reference: images are nx*nx float32 with x fastest
 * (MRC order); a Fourier image is two real arrays (a = Re, b = -Im, the
 * icosprocess/SRC/img2d_FFT.f90:18-19 convention) centred at (nx/2, nx/2).
 */
#ifndef CRYOIM_H
#define CRYOIM_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* ---- status codes ------------------------------------------------------ */
#define CRYOIM_OK            0
#define CRYOIM_ERR_ARG      -1  /* null pointer, non-positive size, bad enum      */
#define CRYOIM_ERR_CUDA     -2  /* a CUDA / cuFFT call failed                      */
#define CRYOIM_ERR_NOMEM    -3  /* device allocation failed                        */
#define CRYOIM_ERR_STATE    -4  /* call order: params / templates not set          */
#define CRYOIM_ERR_SIZE     -5  /* a size is beyond what the kernels support       */
#define CRYOIM_ERR_INPUT    -6  /* NaN/Inf in an input array, bad ort value        */
#define CRYOIM_ERR_IO       -7  /* file missing / short / malformed (host I/O)     */
#define CRYOIM_ERR_MISMATCH -8  /* ort file and stack disagree (checkstckfile)     */

/* ---- records ----------------------------------------------------------- */

/* One particle record, the `particles` type of icosprocess/SRC/0common_icosproc.f90:28-34
 * without its stckfile name (kept by the host I/O layer).  *0 fields hold the values
 * before a search/refinement, d* fields the change, as the reference writes them. */
typedef struct cryoim_particle {
    int32_t particle_id, img_id, img_particle_id;
    float theta0, phi0, omega0, x0, y0, pr0, df1, df2, astigang;
    float theta, phi, omega, x, y, pr;
    float dtheta, dphi, domega, dx, dy, dpr;
} cryoim_particle;

/* One template orientation, the `templates` type of 0common_icosproc.f90:37-40. */
typedef struct cryoim_template {
    int32_t particle_id;
    float theta, phi, omega, x, y;
} cryoim_template;

/* Run parameters: the 32 `key=value` keys of icosprocess/SRC/0input_parameters.f90:6-37
 * that act on this path, their code defaults (0initialvalue.f90:26-45,
 * 0input_parameters.f90:40-51) and the values derived from them
 * (0calc_initialvalues.f90:5-61).  Flags are 0/1 (the reference's 'y'/'n'). */
typedef struct cryoim_params {
    /* inputs */
    int32_t fftsize;        /* FFTsize = nx of the particle stack                  */
    int32_t mode;           /* 1 reconstruct, 4 global search, 5 refinement        */
    int32_t first, last;    /* 1-based particle range                              */
    int32_t ncycle;         /* Ncycle (6)                                          */
    int32_t apply_ctf;      /* applyCTF (y)                                        */
    int32_t use_imgmask;    /* proc2d%imgmask (y)                                  */
    int32_t realspaceavg;   /* realspaceavg (n)                                    */
    int32_t subrec;         /* subrec (n)                                          */
    int32_t fsc;            /* FSC (n)                                             */
    int32_t imgstck;        /* imgstck given (CTF not cached per imgID)            */
    float apix;             /* apix (1.0)                                          */
    float min_res, max_res; /* minRes (300), maxRes (8.0), Angstrom                */
    float imgmask;          /* imgmask, Angstrom ((FFTsize/2-2) before /apix)      */
    float vol, cs, ampwg, bfactor; /* CTF: 300 kV, 2.7 mm, 0.1, 0                  */
    float pr_threshold;     /* PR_threshold (90)                                   */
    float searchstep;       /* searchstep (2.0 degrees)                            */
    float maxcentshift;     /* maxcentshift (100)                                  */
    float boundx;           /* boundX (FFTsize/2-2)                                */
    /* derived by cryoim_params_derive */
    int32_t min_r, max_r;   /* minR=int(apix*N/minRes), maxR=int(apix*N/maxRes) even */
    int32_t nsym, nlin;     /* 60/60 for icos                                      */
    float imgmask_px;       /* mask radius in pixels                               */
    float delta_angle;      /* 360/(maxRes*sqrt(5)*3.14159)                        */
    float delta_trans;      /* FFTsize/(maxRes*sqrt(5))                            */
} cryoim_params;

/* ---- library / context ------------------------------------------------- */

int32_t cryoim_version(void);
/* Text of the last error on this host thread (never NULL). */
const char* cryoim_last_error(void);

/* Fill *p with the reference's code defaults for a stack of nx = fftsize.
 * Replaces icosprocess/SRC/0initialvalue.f90:26-45 and 0input_parameters.f90:40-51. */
int cryoim_params_default(cryoim_params* p, int32_t fftsize);
/* Derive min_r, max_r, imgmask_px, delta_angle, delta_trans, nsym, nlin.
 * Replaces icosprocess/SRC/0calc_initialvalues.f90:4-25 (mode != 6 branch). */
int cryoim_params_derive(cryoim_params* p);

int cryoim_ctx_create(int32_t device, void** ctx_out);
int cryoim_ctx_destroy(void* ctx);
/* Run all device work of this context on `stream` (a cudaStream_t); NULL = own stream. */
int cryoim_ctx_set_stream(void* ctx, void* stream);
/* CUDA-event timing of every launch of the hot kernel (the phase-residual search
 * kernel); off by default.  No reference counterpart (the reference has no timers). */
int cryoim_ctx_set_profiling(void* ctx, int32_t on);
/* Total milliseconds and number of timed launches since the last call (then reset). */
int cryoim_ctx_kernel_time(void* ctx, double* ms, int64_t* launches);
/* Copy and validate parameters (derived fields must be set).  Resets the batch size. */
int cryoim_set_params(void* ctx, const cryoim_params* p);
/* Images processed per device batch (default: min(64, 16M / nx^2)).  No reference
 * counterpart: the reference processes one particle at a time. */
int cryoim_ctx_set_batch(void* ctx, int32_t batch);
/* Pass lanes of the contraction search (1..8, default 6): passes of `batch` particles are
 * dealt round-robin to lanes, each with its own internal stream, device buffers and host
 * thread, so one lane's host work overlaps the others' kernels.  The call stays
 * synchronous: it starts after the work queued on the context's stream and returns when
 * every lane is done.  No reference counterpart. */
int cryoim_ctx_set_lanes(void* ctx, int32_t lanes);

/* ---- templates (icosprocess mode 4/5 set-up) ------------------------------ */

/* Real-space projection of a 3D map (nx^3 float32) along each template orientation
 * by trilinear line integral: replaces icosprocess/SRC/project_template2d.f90:25-76.
 * out: T*nx*nx float32. */
int cryoim_project_templates(void* ctx, const float* map3d, const cryoim_template* t,
                             int32_t T, float* out);
/* Mask, checkerboard, 2D FFT, origin shift and amplitude-cut fit of T template
 * images (T*nx*nx float32); keeps their Fourier transforms resident on the device.
 * Replaces icosprocess/SRC/load_template.f90:35-48. */
int cryoim_load_templates(void* ctx, const float* tmpl_real, const cryoim_template* t,
                          int32_t T);

/* ---- global orientation search (icosprocess mode 4) ------------------------ */

/* Exhaustive search over the icosahedral asymmetric unit scored by the cross-common-
 * line phase residual, for P particles whose images are imgs (P*nx*nx float32, host).
 * parts[] is read (origin, CTF, imgID) and updated in place exactly as
 * icosprocess/SRC/ort_globesearch.f90:34-133 updates particle(i).
 * pr_array (optional, may be NULL): P * Nomega*(2*Nphi+1)*(Ntheta+1) floats, the
 * reference's PR_array(0:Nomega-1,-Nphi:Nphi,0:Ntheta) per particle. */
int cryoim_globesearch(void* ctx, const float* imgs, cryoim_particle* parts, int32_t P,
                       float* pr_array);
/* Same with the images already in device memory (d_imgs, P*nx*nx float32). */
int cryoim_globesearch_device(void* ctx, const float* d_imgs, cryoim_particle* parts,
                              int32_t P, float* pr_array);
/* Grid sizes of the search (ort_globesearch.f90:19-21): Ntheta, Nphi, Nomega and the
 * number of distinct asymmetric-unit views evaluated. */
int cryoim_search_grid(void* ctx, int32_t* ntheta, int32_t* nphi, int32_t* nomega,
                       int32_t* nviews);

/* Phase-residual terms evaluated per particle by the search: sum over views and templates
 * of the valid common lines, times (maxR-minR+1) radii, times Nomega. */
int cryoim_search_terms(void* ctx, double* terms_per_particle);

/* Kernel-level hook: PR(omega) of one particle Fourier image against the loaded
 * templates at view (theta, phi, 0): replaces icosprocess/SRC/cal_crosslin_PR_omega.f90:3-82.
 * ft_a, ft_b: nx*nx (shifted particle FT), fcut0: maxR-minR+1 amplitude cuts of the
 * particle, ctf: nx*nx or NULL (no CTF), pr_omega: Nomega outputs. */
int cryoim_prscore_omega(void* ctx, const float* ft_a, const float* ft_b,
                         const float* fcut0, const float* ctf, float theta, float phi,
                         float* pr_omega);

/* ---- local refinement (icosprocess mode 5) -------------------------------- */

/* Ncycle rounds of the 11-point descent over (theta, phi, omega, x, y) scored by
 * cross-common-line PR.  Replaces icosprocess/SRC/ort_refinement.f90:31-124 with
 * ort_cent_11.f90, return_icos_asymmetry_unit.f90 and cal_crosslin_PR.f90. */
int cryoim_refine(void* ctx, const float* imgs, cryoim_particle* parts, int32_t P);
int cryoim_refine_device(void* ctx, const float* d_imgs, cryoim_particle* parts, int32_t P);
/* Kernel-level hook: PR of one candidate (cal_crosslin_PR.f90:2-71).  ft_a/ft_b is the
 * unshifted particle FT; the candidate origin (x, y) is applied inside. */
int cryoim_prscore(void* ctx, const float* ft_a, const float* ft_b, const float* fcut0,
                   const float* ctf, float theta, float phi, float omega, float x,
                   float y, float* pr);

/* Allocation-free scoring of refinement candidates.  No counterpart in the
 * reference: it exists for callers that cannot allocate device memory when they
 * score (a fixed memory budget owned by another allocator, or a host loop that must
 * not enter the CUDA allocator between steps).  Everything is a caller-owned device
 * pointer and the call runs asynchronously on `stream`; it calls no cudaMalloc,
 * cudaFree or allocating library routine.
 *
 * Computes what cryoim_prscore computes for K <= 11 candidates (theta, phi, omega,
 * x, y) of one particle, from band windows instead of full
 * transforms: a band is the (2*max_r+2)^2 float2 (a, b = -Im) window of a centred
 * nx*nx transform starting at pixel (nx/2-max_r, nx/2-max_r).  d_band: unshifted
 * particle FT; d_fcut0: its max_r-min_r+1 amplitude cuts; d_ctf_band: the particle
 * CTF over the window (NULL = no CTF, then d_tmpl_fcut gives the template cuts);
 * d_tmpl_band: T template windows; d_tmpl_ort: T x (theta, phi, omega); d_pr: K scores.
 *
 * Its intermediate results live in one file-scope device array of about 0.4 MB that
 * every GPU loading the library keeps until the process exits.  Limits: T <=
 * CRYOIM_NOALLOC_MAX_TEMPLATES, K <= CRYOIM_NOALLOC_MAX_CANDIDATES, max_r-min_r+1 <=
 * CRYOIM_NOALLOC_MAX_RADII; larger sizes return CRYOIM_ERR_SIZE.  The first call on a
 * device (with that device current) looks the array up and fills its operator table,
 * a synchronous step: make that first call before any stream capture.  All calls
 * share the one array, so calls that overlap on the GPU (other streams, other host
 * threads) race; serialise them.  The looked-up address and the operator table are
 * kept per device for the life of the process: do not use this entry point across a
 * cudaDeviceReset (or any teardown of the device's primary context).  Errors pending
 * on the calling thread before the call are cleared on entry; a launch failure of this
 * call returns CRYOIM_ERR_CUDA. */
#define CRYOIM_NOALLOC_MAX_TEMPLATES 64
#define CRYOIM_NOALLOC_MAX_CANDIDATES 11
#define CRYOIM_NOALLOC_MAX_RADII 256
int cryoim_prscore_noalloc(int32_t nx, int32_t min_r, int32_t max_r, const float* d_band,
                           const float* d_fcut0, const float* d_ctf_band,
                           const float* d_tmpl_band, const float* d_tmpl_fcut,
                           const float* d_tmpl_ort, int32_t T, const float* d_cand, int32_t K,
                           float* d_pr, void* stream);

/* ---- reconstruction (icosprocess mode 1) --------------------------------- */

/* Start a symmetrised direct-Fourier reconstruction (reconstruct.f90:22-34). */
int cryoim_rec_begin(void* ctx);
/* Insert P particles (host images) whose PR/origin pass the reference's selection
 * (reconstruct.f90:77); returns the number used in *used (may be NULL).
 * Replaces icosprocess/SRC/reconstruct.f90:53-149. */
int cryoim_rec_insert(void* ctx, const float* imgs, const cryoim_particle* parts,
                      int32_t P, int32_t* used);
int cryoim_rec_insert_device(void* ctx, const float* d_imgs, const cryoim_particle* parts,
                             int32_t P, int32_t* used);
/* Friedel completion, divide by the CTF^2 weights, inverse 3D FFT and origin shift
 * into map (nx^3 float32).  Replaces icosprocess/SRC/reconstruct.f90:151-247. */
int cryoim_rec_finish(void* ctx, float* map);
/* Partial accumulators in the tnf half-box layout of reconstruct_substep.f90:18-19,152-155:
 * fa, fb, wg each (2*maxR+1)^2*(maxR+1) floats (x fastest, then y, then z >= 0). */
int cryoim_rec_get_partial(void* ctx, float* fa, float* fb, float* wg);

/* Add a tnf partial (the layout above) into the running accumulator: the summation of
 * merge_icosprocess_subrec/SRC/merge_reconstruct.f90:20-34.  With subrec off, a
 * rec_begin, one add per partial and rec_finish give the merged map. */
int cryoim_rec_add_partial(void* ctx, const float* fa, const float* fb, const float* wg);

/* Start one half map of a gold-standard pair (reconstruct_half.f90:4-151): tnf
 * accumulation with wg starting at 0, samples r <= maxR, boundX from the parameters.
 * The caller inserts the half's particles (first, first+2, ... for the odd half;
 * first+1, first+3, ... for the even half) with cryoim_rec_insert and reads the tnf with
 * cryoim_rec_get_partial.  (mask_x, mask_y): the origin every image is masked at, which
 * in the reference is particle(first) of the whole range for both halves
 * (reconstruct_half.f90:83 passes particle%x).  Replaces the two `call reconstruct_half`
 * of icosprocess/SRC/0main.f90:207-221. */
int cryoim_rec_begin_half(void* ctx, float mask_x, float mask_y);

/* Fourier shell correlation of the odd (fa1, fb1, wg1) and even (fa2, fb2, wg2) tnf half
 * maps and their FSC-weighted sum as a map (reconstruct_FSC.f90:25-178): fsc (maxR+1
 * floats, may be NULL) gets FSC(ir) of the integer shells ir = 0..maxR, as written to
 * FSC.txt; map (nx^3, may be NULL) gets the weighted, Friedel-completed, inverse-FFT map
 * (FFT3d = cmplx(fa, fb) as reconstruct_FSC.f90:173 has it: the point inversion of what
 * reconstruct.f90:241 gives).  Replaces `call reconstruct_fsc` (0main.f90:222). */
int cryoim_fsc_combine(void* ctx, const float* fa1, const float* fb1, const float* wg1,
                       const float* fa2, const float* fb2, const float* wg2, float* fsc,
                       float* map);

/* The FSC merge of merge_icosprocess_subrec (merge_reconstruct_FSC.f90:37-198): the same
 * FSC, weighting and fold as cryoim_fsc_combine on the summed odd and even partials, then
 * the forward-signed transform of that program (Singleton FFT, isn = -1), the
 * (-1)^(x+y+z) shift and a spherical cut at the imgmask radius (params imgmask_px).
 * map: nx^3, before that program's output quirks (which its executable applies). */
int cryoim_merge_fsc_combine(void* ctx, const float* fa1, const float* fb1, const float* wg1,
                             const float* fa2, const float* fb2, const float* wg2, float* fsc,
                             float* map);

/* Finish a summed accumulation (cryoim_rec_add_partial) as merge_reconstruct.f90:37-140
 * does: the Friedel fold keeps int(|h|) <= maxR (its radius is an integer), then the
 * backward transform and origin shift into map (nx^3). */
int cryoim_rec_finish_merge(void* ctx, float* map);

/* Real-space icosahedral average (img3d_icosavg.f90:45-123) of the n^3 host map, in place:
 * voxels with radius > r0 pixels become 0, the others the mean of the map's trilinear
 * samples at the 60 operators' images.  Also applied by cryoim_rec_finish and
 * cryoim_fsc_combine when the parameters ask for realspaceavg (r0 = imgmask_px). */
int cryoim_icosavg(void* ctx, float* map, int32_t n, float r0);

/* ---- origin centring (icosprocess mode 3) -------------------------------- */

/* Re-centre P particles (host images, P x nx^2): with map3d (nx^3, the model) as
 * calc_center.f90:22-105 — each image masked at its origin and Gaussian low-passed
 * (1/e^2 at maxR) is cross-correlated with the model's projection at its orientation
 * (CTF applied when apply_ctf, masked at the centre, low-passed); with map3d NULL as
 * calc_center_selfrot180.f90:22-86 — the image against itself rotated by 180 degrees.
 * A Gaussian fit of the correlation peak gives the new origin (set to 0 beyond nx/16)
 * and PR = acos(peak) in degrees; x0, y0, pr0 keep the old values, dx, dy, dpr the
 * changes; orientations are not touched.  Replaces the mode-3 branch of
 * icosprocess/SRC/0main.f90:237-241. */
int cryoim_center(void* ctx, const float* map3d, const float* imgs, cryoim_particle* parts,
                  int32_t P);

/* ---- localized reconstruction inputs: local_box and local_refine --------- */

/* One sub-particle record: the columns of the local orientation files
 * (local_box/SRC/loc_box_coordinate.f90:35-38 writes the first 23, local_refine reads
 * them in local_refine/SRC/load_original_ort.f90:12-15 and writes all 28 in
 * refine_PR.f90:236-244).  df1, df2 are in Angstrom here (local_box multiplies the
 * micrometre values by 10^4). */
typedef struct cryoim_local_particle {
    int32_t particle_id, img_id, img_particle_id, local_img_id, local_hx0, local_ky0;
    float theta, phi, omega, x, y, pr, df1, df2, astigang;
    float local_theta0, local_phi0, local_omega0, local_x0, local_y0, local_z0, local_pr0;
    float local_theta, local_phi, local_omega, local_x, local_y, local_z, local_pr;
    float local_dtheta, local_dphi, local_domega, local_dx, local_dy;
} cryoim_local_particle;

/* Symmetry rotations of local_box (row-major 3x3 each, at most 60): "cN" (N = 1..60,
 * C_matrix.f90), "i2", "i3", "i5" (icos_matrix_i2.f90, icos_matrix_i3.f90,
 * icos_matrix_i5.f90).  *n receives the count. */
int cryoim_local_sym_matrices(const char* sym, float* out, int32_t* n);

/* local_box's coordinate mode (loc_box_coordinate.f90:13-40) for P whole-particle
 * records (the icosprocess ort fields; selected are those with PR <= pr_threshold and
 * |x|, |y| <= boundx, load_ort.f90:30-34): for every selected particle and every one of
 * the nsym rotations, the equivalent orientation (equalort.f90), the sub-particle
 * centre R^T (loc_x, loc_y, loc_z) + fftsize/2 + (x, y) split into the integer box
 * centre (local_hx0, local_ky0) and the fraction (local_x0, local_y0), and local_z0 =
 * (z - fftsize/2) * apix.  out holds room for P x nsym records; *nout receives the
 * count written. */
int cryoim_local_box_coordinates(const cryoim_particle* parts, int32_t P, const float* sym, int32_t nsym,
                                 float loc_x, float loc_y, float loc_z, float apix, int32_t fftsize,
                                 float pr_threshold, float boundx, cryoim_local_particle* out,
                                 int32_t* nout);

/* local_box's sub-image stack mode (local_box/SRC/loc_box.f90:34-91, selected by
 * local_imgstck=): for each selected particle (PR <= pr_threshold, |x|, |y| <= boundx,
 * load_ort.f90:30-34) of P whole images (imgs: P x fftsize^2 in record order) the image
 * is shifted to centre (img2d_centshift.f90 of local_box at (-x, -y)); for each of the
 * nsym rotations (row-major 3x3) the equivalent orientation (equalort.f90) gives the
 * sub-image centre R^T (loc_x, loc_y, loc_z), and the sub_fftsize^2 box around it is
 * cut with periodic wrap and normalised (img2d_norm.f90).  Outputs, nsym per selected
 * particle in particle order: sub_imgs (room for P x nsym x sub_fftsize^2 floats) and
 * records as loc_box.f90:86-88 writes them: particle_id = the running sub-particle
 * count (format 900's Nparticle), local_img_id = the rotation index, local_theta0..
 * local_omega0 = the equivalent orientation, local_x0 / local_y0 = the fractional part
 * of the centre, local_z0 = its z times apix, local_hx0 / local_ky0 = the box's first
 * pixel, df1 / df2 / astigang as read (micrometres, degrees).  *nout = record count.
 * The whole-image normalisation before the cut (loc_box.f90:47) is not applied: the
 * sub-image normalisation cancels it exactly. */
int cryoim_local_box_extract(void* ctx, const float* imgs, const cryoim_particle* parts, int32_t P, int32_t fftsize,
                             const float* sym, int32_t nsym, float loc_x, float loc_y, float loc_z, float apix,
                             int32_t sub_fftsize, float pr_threshold, float boundx, float* sub_imgs,
                             cryoim_local_particle* out, int32_t* nout);
/* The same with device images in and device sub-images out. */
int cryoim_local_box_extract_device(void* ctx, const float* d_imgs, const cryoim_particle* parts, int32_t P,
                                    int32_t fftsize, const float* sym, int32_t nsym, float loc_x, float loc_y,
                                    float loc_z, float apix, int32_t sub_fftsize, float pr_threshold, float boundx,
                                    float* d_sub_imgs, cryoim_local_particle* out, int32_t* nout);

/* local_refine parameters (local_refine/SRC/0input_parameters.f90:25-55 defaults,
 * 0calc_initialvalue.f90:65-76 derived values). */
typedef struct cryoim_local_params {
    int32_t fftsize;       /* local map box (the sub-particle size)                       */
    int32_t fftsize0;      /* whole-particle image box                                    */
    int32_t nsym;          /* sym cN: N                                                   */
    int32_t ncycle;        /* refinement cycles (12)                                      */
    int32_t apply_ctf;     /* 1 (applyCTF=y)                                              */
    int32_t normalize;     /* 1: img2d_norm of the whole image (stack files); 0 (imgstck)  */
    float apix, max_res, imgmask, vol, cs, ampwg, refine_angle, refine_shift, convf;
    /* derived by cryoim_local_params_derive: */
    float max_r;           /* apix * fftsize / max_res (pixels, not rounded)              */
    float imgmask_px;      /* imgmask / apix if imgmask > 0, else fftsize/2 - 2            */
} cryoim_local_params;

/* The reference defaults (apix 1, maxRes 10, Ncycle 12, convF 0.8, vol 200, Cs 2.7,
 * ampwg 0.1, sym c1, applyCTF y, refine_angle / refine_shift derived when <= 0). */
int cryoim_local_params_default(cryoim_local_params* p, int32_t fftsize, int32_t fftsize0);
int cryoim_local_params_derive(cryoim_local_params* p);

/* local_refine's refine_PR (refine_PR.f90:55-232) for P sub-particles: whole-particle
 * images (P x fftsize0^2, one per record, in record order), the local map
 * (fftsize^3).  Each sub-particle is boxed at (local_hx0, local_ky0), masked at its
 * (local_x0, local_y0), transformed and Gaussian-weighted; with nsym > 1 the nsym
 * equivalent orientations (icos_equalort) are scored first, then ncycle rounds of the
 * 11-candidate descent, every candidate scored by cal_PR_FT against the map's central
 * section (FFT3d_slice) shifted to the candidate origin, times CTF and the weight.  The
 * local_* output fields are set as refine_PR.f90:220-231 sets them. */
int cryoim_local_refine(void* ctx, const cryoim_local_params* p, const float* map3d, const float* imgs,
                        cryoim_local_particle* parts, int32_t P);

/* The local orientation files: 23 list-directed columns in, and out either the 23 of
 * local_box (format 900 of loc_box_coordinate.f90:46, columns = 23), the 28 of
 * local_refine (format 901 of refine_PR.f90:246-253, columns = 28) or the 14 of
 * local_box's sub-image stack mode (format 900 of loc_box.f90:93, columns = 14).  stck as in
 * cryoim_ort_read (stck_len bytes per record, name width 64 on output). */
int cryoim_local_ort_read(const char* path, int32_t first, int32_t last, cryoim_local_particle* parts,
                          char* stck, int32_t stck_len);
int cryoim_local_ort_write(const char* path, const cryoim_local_particle* parts, const char* stck,
                           int32_t stck_len, int32_t n, int32_t columns, int32_t append);

/* ---- files (host only; byte-compatible with the reference) ---------------- */

/* The `mrchead` type of icosprocess/SRC/0common_icosproc.f90:61-112: 1024 bytes. */
typedef struct cryoim_mrc_header {
    int32_t nx, ny, nz, mode, nxstart, nystart, nzstart, mx, my, mz;
    float a, b, c, alpha, beta, gamma;
    int32_t mapc, mapr, maps;
    float amin, amax, amean;
    int32_t ispg, nsymbt, extra[25];
    float xorigin, yorigin, zorigin;
    char map[4], machinestamp[4];
    float arms;
    int32_t nlabl;
    char label[800];
} cryoim_mrc_header;
int cryoim_mrc_read_header(const char* path, cryoim_mrc_header* h);
/* count images (sections) starting at the 1-based index first, float32 (mode 2) only */
int cryoim_mrc_read_sections(const char* path, int32_t first, int32_t count, float* out);
/* mrchead.f90:2-58 (maphead) for an nx x ny x nz float map */
int cryoim_map_header(cryoim_mrc_header* h, int32_t nx, int32_t ny, int32_t nz, float apix);
int cryoim_mrc_write(const char* path, const cryoim_mrc_header* h, const float* data, int64_t n);
/* non-blank rows of an orientation file */
int cryoim_ort_count(const char* path, int32_t* n);
/* rows first..last (1-based) of a 13-column orientation file (load_original_ortcent.f90);
 * stck (optional): (last-first+1) x stck_len bytes of stack names */
int cryoim_ort_read(const char* path, int32_t first, int32_t last, cryoim_particle* parts,
                    char* stck, int32_t stck_len);
/* name_width 54: the 19-column row of format 900 (ort_globesearch.f90:139);
 * name_width 64: proc_icos's 13-column row (transform_ort_2fTo5f.f90:36) */
int cryoim_ort_write(const char* path, const cryoim_particle* parts, const char* stck,
                     int32_t stck_len, int32_t n, int32_t name_width, int32_t append);
/* template orientation rows `id theta phi omega x y` (load_template.f90:18-21); *n = rows */
int cryoim_template_ort_read(const char* path, cryoim_template* t, int32_t maxn, int32_t* n);
/* tnf partial (reconstruct_substep.f90:152-155) */
int cryoim_tnf_write(const char* path, int32_t fftsize, int32_t max_r, float apix, float imgmask,
                     int32_t flag_fsc, int32_t flag_avg, const float* fa, const float* fb,
                     const float* wg);
/* ihdr[4] = fftsize, max_r, flag_fsc, flag_avg; fhdr[2] = apix, imgmask; arrays optional */
int cryoim_tnf_read(const char* path, int32_t* ihdr, float* fhdr, float* fa, float* fb, float* wg);

/* ---- central sections (projection-matching form, spec step a/b) ------ */

/* Trilinear central sections of a 3D Fourier map: replaces
 * icosprocess/SRC/project2d_FT3dTo2d.f90:19-84 (the section before its inverse FFT).
 * ft_re/ft_im: nx^3 float32 (x fastest, centred at nx/2); eulers: n*3 (theta,phi,omega)
 * degrees; out_re/out_im: n*nx*nx float32. */
int cryoim_central_sections(void* ctx, const float* ft_re, const float* ft_im,
                            const float* eulers, int32_t n, float* out_re, float* out_im);

/* ---- projection-matching contraction form -------------------------------- */
/* No counterpart in the reference, which scores by phase residual only.  A second
 * search beside cryoim_globesearch: the cross-correlation of every (particle, origin)
 * with every grid orientation's central section, run as one dense BF16 contraction on
 * the tensor cores (FP32 accumulation); per particle the best origin of every block of
 * 256 orientations is kept and the top-k of those (distinct orientations) are rescored
 * in FP64.  pick = 0 (drop-in for mode 4): each candidate orientation and its 26 grid
 * neighbours are scored with the reference's phase residual (cal_crosslin_PR.f90) at
 * the particle's own origin, as ort_globesearch.f90 scores every view, and the minimum
 * is taken; the origin is left unchanged.  pick = 1: the candidate with the largest FP64
 * cross-correlation, orientation and origin. */
typedef struct cryoim_contract_opts {
    float origin_max;   /* origins searched on [-origin_max, origin_max]^2 pixels   */
    float origin_step;  /* origin grid step, pixels                                 */
    int32_t topk;       /* candidates rescored per particle (1..64)                 */
    int32_t pick;       /* 0: minimum phase residual, 1: maximum FP64 correlation  */
    int32_t precision;  /* operands: 0 BF16, 1 FP8-e4m3 with per-band power-of-two
                           scales (both with FP32 accumulation)                    */
    int32_t nbr;        /* PR rescoring of each candidate's grid neighbours within
                           nbr steps in theta, phi and omega (1: 26 neighbours; 0 is
                           taken as 1); (2 nbr + 1)^3 x topk <= 4096                 */
    int32_t coarse;     /* 0: every grid orientation is correlated.  k > 0 (<= 64):
                           proposal form: a BF16 contraction over half the band, a
                           grid of twice the step and origins at twice the step names
                           k orientations; only their fine neighbourhoods (+-2 steps,
                           proposal_nbr) are correlated at full band                */
    int32_t learned;    /* 0: off.  k > 0 (<= 64, not with coarse): the trained
                           proposer (cryoim_learn_train / _load) names k cells (view
                           of the twice-the-step grid, in-plane angle and the angle
                           + 180 degrees) per particle; their fine neighbourhoods
                           (+-2 steps) are correlated as in the coarse form           */
    int32_t nbr_best;   /* 0: the phase-residual rescoring covers the neighbourhoods of
                           all topk candidates.  m > 0: the candidates are scored
                           first, then only the neighbourhoods of the m with the least
                           phase residual                                            */
    float local_range;  /* 0: global search.  > 0: local search of each particle around
                           its own (theta, phi, omega): every grid point theta + i s,
                           phi + j s, omega + k s, |i|, |j|, |k| <= round(local_range / s),
                           s = local_step (degrees), against every origin; the sections
                           of these orientations are cut from the map's band cube for
                           the pass and correlated in BF16 on the tensor cores, the topk
                           best rescored in FP64 (pick = 1, precision = 0, no coarse or
                           learned proposals, no templates needed; at most 2,146,689
                           orientations per particle).  The local form of sub-particle
                           refinement; no reference counterpart                      */
    float local_step;
    float fallback;     /* learned form only.  0: off.  t > 0: run-time fallback to the
                           exhaustive contraction: after the learned form, every
                           particle whose phase residual exceeds the call's median by
                           more than t robust standard deviations (1.4826 x the median
                           absolute deviation) is searched again by the exhaustive
                           BF16 contraction with the same options, and the result of
                           lower phase residual is kept (pick = 0).  The count is
                           returned by cryoim_contract_fallbacks                     */
    int32_t centred_origins; /* 0: the origin grid is absolute.  1: it is centred on
                           each particle's own (x, y) (the local form's re-centred
                           origin search; PR rescoring is unaffected)                */
    int32_t proposal_nbr; /* coarse and learned forms: each proposal's fine
                           neighbourhood, +-proposal_nbr steps in theta, phi and
                           omega (0 is taken as 2; 1..4)                             */
} cryoim_contract_opts;

/* ---- learned orientation proposer ------------------------------------------- */
/* A small rotation-equivariant CNN on each particle's polar power spectrum (64 radii
 * over [minR, maxR] x 128 angles over half a turn): four 3x3 convolutions circular in
 * angle, a (channel, radius) mix to 16 channels per angle, and one learned template
 * per view of the twice-the-search-step grid scored at every circular angle shift.
 * Trained on projections the library renders from the map (real-space projector, CTF,
 * origin shift, white noise), labelled with their orientations folded into the
 * asymmetric unit.  No counterpart in the reference. */
typedef struct cryoim_learn_opts {
    int32_t samples;    /* training projections (default 200000)                    */
    int32_t batch;      /* minibatch (default 256)                                  */
    int32_t seed;       /* orientations, CTF, origins, noise and initial weights    */
    float lr;           /* Adam learning rate (default 2e-3)                        */
    float snr;          /* signal / noise variance inside the 0.4 nx disc (0: none) */
    float df_min, df_max;   /* defocus range, um                                    */
    float astig_max;    /* astigmatism up to this (um) at a uniform angle           */
    float origin_max;   /* origins uniform on [-origin_max, origin_max]^2 px        */
} cryoim_learn_opts;
int cryoim_learn_opts_default(cryoim_learn_opts* o);
/* Trains (or retrains) the proposer of ctx for its parameters' search step.  map3d:
 * nx^3 real map on the host, from which the training particles are rendered
 * (cryoim_learn_render).  stats (may be NULL) <- [mean loss of the last 10% of
 * steps, seconds, angle sign (+1 / -1), views]. */
int cryoim_learn_train(void* ctx, const float* map3d, const cryoim_learn_opts* o, float* stats);
/* The trained weights to / from a file (little-endian: "CRYOIMLP", version, views,
 * angle sign, search step, parameter count, FP32 parameters). */
int cryoim_learn_save(void* ctx, const char* path);
int cryoim_learn_load(void* ctx, const char* path);
/* Test hooks: parameters (get and / or set; *n <- count), and one forward (+ backward
 * with truth) on given features [B][64][128]: scores [B][views][128], loss per
 * particle [B], parameter gradients (NULL to skip).  truth[b] = (view unit vector,
 * angle shift). */
int cryoim_learn_params(void* ctx, float* get, const float* set, int64_t* n);
int cryoim_learn_forward(void* ctx, const float* feat, const float* truth, int32_t B, float* scores,
                         float* loss, float* grads);
/* Arithmetic of the proposer's 3x3 convolutions (training and inference): 1 (default):
 * tcgen05 tensor cores, operands rounded to TF32 (10 mantissa bits, to nearest, ties
 * away from zero), FP32 accumulation; 0: FP32 on the CUDA cores. */
int cryoim_learn_set_conv(void* ctx, int32_t tensor_cores);
/* Test hook of the convolution kernels on host arrays (current device): x [B][Cin][H][128],
 * W [Cout][Cin][3][3], bias [Cout] (may be NULL) -> out [B][Cout][H][128] (circular in the
 * 128 angles, zero-padded in H, ReLU if relu); with dpre [B][Cout][H][128] also the weight
 * and bias gradients dW, db.  Cin <= 32 (1 or a multiple of 8 with dpre), Cout 16 or 32. */
int cryoim_conv3_check(int32_t tensor_cores, const float* x, int32_t B, int32_t Cin, int32_t H, const float* W,
                       const float* bias, int32_t Cout, int32_t relu, float* out, const float* dpre, float* dW,
                       float* db);
/* The proposer's training renderer: B particles of the nx^3 map (host) at eul[b] =
 * (theta, phi, omega) with par[b] = (df1, df2, astig, x, y) (CTF if apply_ctf), white
 * noise at snr (0: none) from seed -> imgs [B][nx][nx].  Fourier slices of the twice
 * zero-padded map's transform, low-passed at maxR + 1. */
int cryoim_learn_render(void* ctx, const float* map3d, const float* eul, const float* par, int32_t B, float snr,
                        int32_t seed, float* imgs);
/* The proposer's classes: views (theta, phi) of the twice-the-step grid, in order
 * (out may be NULL; *V <- count). */
int cryoim_learn_views(void* ctx, float* out, int32_t* V);
/* The proposer's input features [P][64][128] of P particles (mask at each particle's
 * origin, transform, polar power spectrum). */
int cryoim_learn_features(void* ctx, const float* imgs, const cryoim_particle* parts, int32_t P,
                          float* feat);
/* The 3D map (nx^3 float32) whose central sections are correlated: its centred Fourier
 * transform is kept as a band cube of (2 maxR + 3)^3 complex values. */
int cryoim_set_reference_map(void* ctx, const float* map3d);
/* cands (optional): P x topk x 8 floats: theta, phi, omega, x, y (the candidate's best
 * origin), CC from the contraction (BF16 or FP8), CC in FP64, PR at the particle's origin. */
int cryoim_contract_search(void* ctx, const float* imgs, cryoim_particle* parts, int32_t P,
                           const cryoim_contract_opts* opts, float* cands);
int cryoim_contract_search_device(void* ctx, const float* d_imgs, cryoim_particle* parts, int32_t P,
                                  const cryoim_contract_opts* opts, float* cands);
/* Interpolation of the central sections the contraction forms cut from the reference
 * map (the BF16/FP8 section bank, the local grids and the FP64 rescoring): kind 0
 * trilinear (the default, as project2d_FT3dTo2d.f90:30-83 interpolates), kind 1 a
 * Gaussian kernel: the 27 voxels around the nearest one, weighted exp(-d^2/(2 sigma^2)),
 * normalised by the weights' sum (sigma 0.25..2 voxels), kind 2 trilinear on the
 * transform of the map zero-padded to twice its side (a twice-oversampled transform: 8x
 * the 3D FFT and its band cube; sections match the map's projections to a correlation of
 * ~0.998 instead of ~0.96, which keeps the interpolation error from moving a local
 * search's maximum).  The reference has trilinear interpolation only.  Changing it
 * rebuilds the band cube (kind 2 <-> 0/1) and the section bank at the next search. */
int cryoim_set_interpolation(void* ctx, int32_t kind, float sigma);
/* Particles the last call of a contraction search sent to the exhaustive fallback
 * (cryoim_contract_opts.fallback). */
int cryoim_contract_fallbacks(void* ctx, int32_t* n);
/* out[6]: section build ms, contraction ms and launches since the last call (timed when
 * profiling is on), contraction FLOP, orientations, padded K. Resets the counters. */
int cryoim_contract_stats(void* ctx, double* out);
/* out[3]: the contraction forms' phase-residual rescoring since the last call (timed when
 * profiling is on): launch ms, launches, candidates scored.  Resets the counters. */
int cryoim_rescore_stats(void* ctx, double* out);

/* Kernel-level hook of the tensor-core contraction (no reference counterpart: the
 * reference has no cross-correlation search).  Device pointers: A (M x K) and B (N x K)
 * BF16 row-major with K % 64 == 0; C = A B^T in FP32 is reduced to the max and argmax
 * of every (row, 256-column tile): d_topv / d_topi are M x ceil(N/256); d_c (optional)
 * receives the full M x N C.  *d_err = 1 if a pipeline wait timed out. */
int cryoim_gemm_bf16_argmax(const void* d_a, const void* d_b, int32_t M, int32_t N, int32_t K,
                            float* d_topv, int32_t* d_topi, float* d_c, int32_t* d_err,
                            void* stream);
/* The same with FP8-e4m3 operands (one byte per element, K % 128 == 0), FP32 accumulation
 * (tcgen05.mma kind::f8f6f4). */
int cryoim_gemm_e4m3_argmax(const void* d_a, const void* d_b, int32_t M, int32_t N, int32_t K,
                            float* d_topv, int32_t* d_topi, float* d_c, int32_t* d_err,
                            void* stream);
/* Test of the contraction kernel's failure path (device pointers as above, no full C):
 * CTA 0 leaves k-stage `stage` (0 <= stage < K / 64) of its first tile unloaded, so the
 * MMA issuer's wait for that stage cannot complete; every wait of the launch gives up
 * after wait_us microseconds (100 .. 2,000,000).  *d_err is 1 afterwards, the kernel has
 * returned with its TMEM released, and the next launch works.  No reference counterpart. */
int cryoim_gemm_bf16_argmax_withhold(const void* d_a, const void* d_b, int32_t M, int32_t N, int32_t K,
                                     float* d_topv, int32_t* d_topi, int32_t* d_err, int32_t stage,
                                     int32_t wait_us, void* stream);

/* ---- orientation bookkeeping (proc_icos) --------------------------------- */

/* The 60 icosahedral rotations in the 2-fold frame, in the order of
 * icosprocess/SRC/icos2f_sym_mat.f90:5-243 (rot[k*9 + r*3 + c]). */
int cryoim_icos_ops(float* rot);
/* Fold an orientation into the asymmetric unit (return_icos_asymmetry_unit.f90:1-33). */
int cryoim_asu_fold(float* theta, float* phi, float* omega);
/* The 60 symmetry-equivalent orientations (proc_icos/SRC/equalort.f90:1-24): out 60*3. */
int cryoim_equalort(float theta, float phi, float omega, float* out);
/* 2-fold -> 5-fold (to=5) or 2-fold -> 3-fold (to=3) frame, in place on n orientations
 * (proc_icos/SRC/transform_ort_2fTo5f.f90:11-30, transform_ort_2fTo3f.f90:11-32). */
int cryoim_transform_ort(int32_t to, float* theta, float* phi, float* omega, int32_t n);

#ifdef __cplusplus
}
#endif
#endif /* CRYOIM_H */
