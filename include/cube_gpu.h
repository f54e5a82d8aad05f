/*
 * cube_gpu.h -- C ABI of the GB300 implementation of CUBE's per-step
 * gravity/update path (drift + counting re-sort, PP kick, two-level PM kick).
 *
 * Each entry point replaces the body of one reference subroutine; the
 * Fortran driver (CUBEnu/work/main/main.f90:88-145) keeps its loop and binds
 * these functions with iso_c_binding.  All particle and mesh state stays
 * resident in device memory between calls; host pointers are borrowed only
 * for the duration of a call.  Every call returns an int status (CUBE_OK=0),
 * replacing the reference's `stop` statements; cube_last_error() gives text.
 * Threading: one CUDA stream per context, calls on one context must not
 * overlap; independent contexts are independent.
 *
 * Array layouts are the reference's (Fortran, first index fastest):
 *   xp(3,np)  int8 (izipx=1) or int16 (izipx=2)   variables.f90:44
 *   vp(3,np)  int8 (izipv=1) or int16 (izipv=2)   variables.f90:45
 *   pid(np)   int32                               variables.f90:47
 *   rhoc(nt,nt,nt,nnt,nnt,nnt) int32  physical counts (checkpoint.f90:42)
 *   vfield(3,nt,nt,nt,nnt,nnt,nnt) float          (checkpoint.f90:44)
 * Particles are in the reference's disjoint order: tile (x fastest), then
 * coarse cell (x fastest) inside the tile, then rank in cell
 * (update_particle.f90:132-142).
 */
#ifndef CUBE_GPU_H
#define CUBE_GPU_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* Status codes; each replaces a `stop` of the reference. */
enum cube_status {
  CUBE_OK = 0,
  CUBE_ERR_ARG = 1,             /* bad argument or size */
  CUBE_ERR_CUDA = 2,            /* CUDA / cuFFT failure */
  CUBE_ERR_TILE_OVERFLOW = 3,   /* update_particle.f90:88-94 */
  CUBE_ERR_IMAGE_OVERFLOW = 4,  /* buffer_grid.f90:148-154: particle capacity exceeded */
  CUBE_ERR_PP_OVERFLOW = 5,     /* ext_pp_force.f90:41-45 */
  CUBE_ERR_COUNT_MISMATCH = 6,  /* ext_pp_force.f90:156-160, update_particle.f90:245-250 */
  CUBE_ERR_NONFINITE = 7,       /* a force or velocity became NaN/Inf */
  CUBE_ERR_DISPLACEMENT = 8,    /* a particle left the double-buffer tile
                                   (update_particle.f90:71 would index out of bounds) */
  CUBE_ERR_NOMEM = 9,
  CUBE_ERR_STATE = 10           /* call out of order (e.g. no state uploaded) */
};

/* Run-time image of the Fortran `parameter`s (parameters.f90:8-65). */
typedef struct cube_params {
  int32_t nc;         /* coarse cells per dim (nc) */
  int32_t nnt;        /* tiles per dim (nnt); nt = nc/nnt */
  int32_t ncell;      /* fine cells per coarse cell per dim (4) */
  int32_t ncb;        /* buffer depth in coarse cells (6) */
  int32_t izipx;      /* bytes per stored position component (1|2) */
  int32_t izipv;      /* bytes per stored velocity component (1|2) */
  int32_t nf_cutoff;  /* fine force table extent (16) */
  int32_t pp_range;   /* PP neighbourhood in fine cells (1) */
  int32_t pp_on;      /* Extended_pp_force */
  int32_t with_pid;   /* -DPID: carry particle ids */
  float rsoft;        /* PP hard cut radius, fine cells */
  float mass_p;       /* sim%mass_p_cdm */
  int64_t np_max;     /* particle capacity of the device arrays */
  int32_t reserved[8];
} cube_params;

/* Scalars each call returns (the reference prints or stores these). */
typedef struct cube_stats {
  /* cube_update_x (update_particle.f90:16-256) */
  int64_t nplocal;        /* sim%nplocal after the re-sort */
  int64_t max_tile_np;    /* largest double-buffer tile count (overhead_tile numerator) */
  int64_t nlost;          /* particles that landed in no physical cell */
  int64_t ndup;           /* extra copies (landed in two frames) */
  double sum_c, sum_r, sum_s; /* sigma_v sums (update_particle.f90:172-196) */
  float sigma_vi_new;     /* std_vsim_res/sqrt(3.) */
  int32_t nlayer;         /* layer count used for the visit order */
  int32_t max_disp;       /* largest cell displacement seen */
  int32_t rank_walked;    /* ranks came from 0: the counting path, 1: the walker, 2: the sort */
  /* cube_pp_force (ext_pp_force.f90:10-162) */
  float f2_max_pp;
  int32_t pp_dense_bricks; /* bricks redone cell by cell (too dense to stage) */
  int64_t npairs;
  int64_t itest1;
  /* cube_particle_mesh (pm.f90:2-415) */
  float f2_max_fine;
  float f2_max_coarse;
  float vmax[3];
  int32_t pad2;
  double testrhof, testrhoc;
  int32_t flags;
  int32_t pad3;
} cube_stats;

/* The reference's checkpoint header, type sim_header (parameters.f90:136-160),
   byte for byte as Fortran stream I/O writes it: 17 int64 then 22 real(4). */
typedef struct cube_sim_header {
  int64_t nplocal, npglobal, nplocal_nu, npglobal_nu;
  int64_t izipx, izipv, izipx_nu, izipv_nu;
  int64_t image;
  int64_t nn, nnt, nt, ncell, ncb;
  int64_t timestep;
  int64_t cur_checkpoint;
  int64_t cur_halofind;
  float a, t, tau;
  float dt_pp, dt_fine, dt_coarse, dt_vmax, dt_vmax_nu;
  float mass_p_cdm, mass_p_nu;
  float box;
  float h0, omega_m, omega_l, s8;
  float vsim2phys, sigma_vres, sigma_vi, sigma_vi_nu;
  float z_i, z_i_nu;
  float vz_max;
} cube_sim_header;

/* Cosmology and particle grid of the initial conditions. */
typedef struct cube_cosmology {
  float box;       /* Mpc/h */
  float omega_m, omega_l, h0, s8, n_s;
  float omega_b;   /* baryon fraction of the Eisenstein-Hu no-wiggle shape */
  int32_t np_nc;   /* particles per coarse cell per dimension */
} cube_cosmology;

typedef struct cube_ctx cube_ctx;

/* Fields for inspection / injection in parity tests. */
enum cube_field {
  CUBE_FIELD_RHO_F = 1,    /* fine density, nf^3 float, global periodic, Fortran order */
  CUBE_FIELD_FORCE_F = 2,  /* fine force, 3 planes of nf^3 float (x, y, z) */
  CUBE_FIELD_RHO_C = 3,    /* coarse density nc^3 float */
  CUBE_FIELD_FORCE_C = 4,  /* coarse force, 3 planes of nc^3 float */
  CUBE_FIELD_KERN_F = 5,   /* fine kernel Im part, 3 planes of (nf/2+1)*nf*nf float (unscaled) */
  CUBE_FIELD_KERN_C = 6,   /* coarse kernel, 3 planes of (nc/2+1)*nc*nc float (unscaled) */
  CUBE_FIELD_FORCE_PP = 7  /* PP pair force of the last cube_pp_force, f_tot(3,nplocal) float in
                              storage order (ext_pp_force.f90:94-112); read-only */
};

/* Build a context on `device`: allocates every device buffer for the given
   sizes and builds the fine and coarse Green's functions from the force
   tables (replaces initialize + kernel_f + kernel_c, initialize.f90:21-38,
   kernel_f.f90:14-37, kernel_c.f90:16-117).
   fine_table: fk_table(i,j,k,d), 16x16x16x3 float, Fortran order.
   coarse_table: ck_table(d,i,j,k), 3x4x4x4 float, Fortran order.
   Sizes rejected with CUBE_ERR_ARG before any device call (the message in
   cube_last_error): nc outside 16..16384 or not a multiple of nnt, ncell
   other than 4, izipx/izipv outside 1..2, nc/nnt below 2*ncb, ncb outside
   1..8, nf_cutoff not below ncb*ncell, pp_range other than 1 with PP on,
   np_max not positive. */
int cube_create(const cube_params* p, const float* fine_table, const float* coarse_table, int device,
                cube_ctx** out);
int cube_destroy(cube_ctx* ctx);

/* A second particle species (CUBEnu's neutrinos, initialize.f90:90-136): a
   context with its own compressed state, codec and sigma_vi (p gives its
   izipx/izipv, mass_p and np_max; the mesh geometry must equal the owner's,
   pp_on must be 0) that shares the owner's meshes, force kernels, FFT plans
   and stream.  Destroy it before its owner.  cube_update_x, the checkpoint
   calls (files named *_nu) and cube_power_spectrum work on it as on any
   context; cube_particle_mesh2 advances both species together. */
int cube_create_linked(const cube_params* p, cube_ctx* owner, cube_ctx** out);
const char* cube_last_error(const cube_ctx* ctx);

/* Upload / download the disjoint state (particle_initialization.f90:34-78,
   checkpoint.f90:36-47).  nplocal <= np_max. pid may be NULL. */
int cube_upload_state(cube_ctx* ctx, int64_t nplocal, const void* xp, const void* vp, const int32_t* pid,
                      const int32_t* rhoc, const float* vfield);
int cube_download_state(cube_ctx* ctx, int64_t* nplocal, void* xp, void* vp, int32_t* pid, int32_t* rhoc,
                        float* vfield);

/* Upload and download overlapped with the step, for a driver that keeps the
   state in host memory and moves it every step.  Host memory should be
   page-locked for the copies to run asynchronously.

   cube_upload_begin is cube_upload_state with vfield, xp, vp and pid copied
   on a side stream, xp and vp in four pieces: the counts are checked before
   it returns (they need only rhoc), the re-sort's first pass takes each
   piece of xp and vp as it lands, and the re-sort reads pid only in its
   scatter.  The host xp, vp and pid arrays must stay unchanged until the
   next cube_update_x (or cube_synchronize) returns; any other call that
   reads the state first waits for the whole upload.

   cube_download_begin, called after cube_update_x and the buffer calls,
   starts copying xp, pid, rhoc and vfield, which are final for the step (PP
   and PM read them and write only vp), on a side stream and returns.  vp is
   copied behind the next coarse kick, piece by piece as the kick finishes
   each eighth of the particles, or by cube_download_finish when no kick
   comes first.  cube_download_finish returns when all of them are in host
   memory.  Any array may be NULL.  A call that changes the state before the
   finish (cube_update_x, an upload, a checkpoint read, initial conditions)
   is ordered after the copies on the device. */
int cube_upload_begin(cube_ctx* ctx, int64_t nplocal, const void* xp, const void* vp, const int32_t* pid,
                      const int32_t* rhoc, const float* vfield);
int cube_download_begin(cube_ctx* ctx, int64_t* nplocal, void* xp, void* vp, int32_t* pid, int32_t* rhoc,
                        float* vfield);
int cube_download_finish(cube_ctx* ctx);

/* Checkpoint files in the reference's format (checkpoint.f90:10-50; read back
   as particle_initialization.f90:34-64 does): in dir, <z>_info_<image>.bin,
   _xp_, _vp_, _np_, _vc_ and (with particle ids) _id_, <z> = z printed as
   Fortran f7.3 without blanks.  Write fills nplocal, izipx/v, nnt, nt, ncell,
   ncb, image and sigma_vi from the context -- and, when a second species is
   linked to the context and holds a state, nplocal_nu, izipx_nu, izipv_nu
   and sigma_vi_nu from that species (checkpoint.f90:31-32) -- and takes the
   other header fields from hdr; read checks the zip format and tile geometry, uploads the state,
   sets sigma_vi and returns the header in hdr (may be NULL).  On a linked
   context (the second species) they use the _xp_nu_, _vp_nu_, _np_nu_,
   _vc_nu_, _id_nu_ files, write no info file, and read nplocal_nu, izipx_nu,
   izipv_nu and sigma_vi_nu from the owner's info file. */
int cube_checkpoint_write(cube_ctx* ctx, const char* dir, float z, int image, const cube_sim_header* hdr);
int cube_checkpoint_read(cube_ctx* ctx, const char* dir, float z, int image, cube_sim_header* hdr);

/* Zel'dovich initial conditions generated on the device into the context's
   state (initial_conditions.f90:250-825, with an Eisenstein-Hu no-wiggle
   transfer function and a counter-hash white noise): (nc*np_nc)^3 particles
   at z_init in the compressed layout, particles of a cell in Lagrangian order.
   Returns sigma_vi (also set in the context) and the largest |v| per
   dimension.  Uses the fine-mesh buffers as scratch. */
int cube_ic_zeldovich(cube_ctx* ctx, const cube_cosmology* cosmo, float z_init, uint32_t seed, float* sigma_vi,
                      float* vmax);
/* The same for a massive-neutrino species (CUBEnu; replaces the thermal part
   of CUBEnu/initial_conditions_mnu.f90:95-115): each particle's Zel'dovich
   velocity plus an isotropic thermal velocity of speed q * 50.2476 km/s /
   m_nu[eV] / a, q drawn from the relativistic Fermi-Dirac distribution
   q^2/(e^q+1) by inverse CDF, in simulation units (vsim2phys of
   initial_conditions.f90:175).  seed sets the density field (give the
   CDM's seed for the same field), thermal_seed the thermal draws. */
int cube_ic_zeldovich_nu(cube_ctx* ctx, const cube_cosmology* cosmo, float z_init, uint32_t seed, float m_nu_ev,
                         uint32_t thermal_seed, float* sigma_vi, float* vmax);

/* sigma_vi / sigma_vi_new module variables (variables.f90:36). */
int cube_set_sigma(cube_ctx* ctx, float sigma_vi, float sigma_vi_new);
int cube_get_sigma(const cube_ctx* ctx, float* sigma_vi, float* sigma_vi_new);

/* update_x -> update_xp (update_particle.f90:5-256): drift by
   dt_mid=(dt_old+dt)/2, counting re-sort in the reference's layered visit
   order, new rhoc/vfield, sigma_v statistics; sets sigma_vi_new.
   vz_max is sim%vz_max (pm.f90:398). */
int cube_update_x(cube_ctx* ctx, float dt_old, float dt, float vz_max, cube_stats* st);

/* buffer_grid / buffer_x / buffer_v (buffer_grid.f90:5-26,
   buffer_particle.f90:5-25): the device kernels index the periodic
   neighbours directly, so these only validate the context. */
int cube_buffer_grid(cube_ctx* ctx);
int cube_buffer_x(cube_ctx* ctx);
int cube_buffer_v(cube_ctx* ctx);

/* ext_pp_force (ext_pp_force.f90:10-162): pair force within +-pp_range fine
   cells with the hard cut rsoft, kick v by F*a_mid*dt/(6 pi). */
int cube_pp_force(cube_ctx* ctx, float a_mid, float dt, cube_stats* st);

/* particle_mesh (pm.f90:2-415): fine PM kick (decode sigma_vi, encode
   sigma_vi_new), then sigma_vi=sigma_vi_new, then coarse PM kick; returns
   the force maxima and vmax. */
int cube_particle_mesh(cube_ctx* ctx, float a_mid, float dt, cube_stats* st);

/* cube_pp_force followed by cube_particle_mesh (main.f90:113-116) in one
   call: PP runs on a second stream beside the PM densities, transforms and
   maxima (they read positions only), and the fine kick waits for PP's kick.
   Bit for bit the results of the two calls in sequence; st_pp receives PP's
   stats, st_pm particle_mesh's. */
int cube_pp_particle_mesh(cube_ctx* ctx, float a_mid, float dt, cube_stats* st_pp, cube_stats* st_pm);

/* particle_mesh of two species (pm.f90:52-107, 162-194, 237-253, 358-377):
   the linked species nu deposits into the same meshes with its own mass, both
   are kicked by the same forces with their own velocity codes, sigma_vi and
   vmax (st_nu). */
int cube_particle_mesh2(cube_ctx* ctx, cube_ctx* nu, float a_mid, float dt, cube_stats* st, cube_stats* st_nu);
/* Its density stages, for parity tests: both species deposited into the
   shared fine (coarse) mesh, each cell's second-species particles after the
   first's (pm.f90:52-107 / 205-267); st->testrhof (testrhoc) is the total. */
int cube_pm_fine_density2(cube_ctx* ctx, cube_ctx* nu, cube_stats* st);
int cube_pm_coarse_density2(cube_ctx* ctx, cube_ctx* nu, cube_stats* st);

/* Stages of particle_mesh, for parity tests that inspect or inject fields:
   density only (CIC deposit, pm.f90:52-107 / 205-267), forces (deposit +
   Green's multiply + inverse FFT; the density buffer then holds the
   spectrum) and kick only. */
int cube_pm_fine_density(cube_ctx* ctx, cube_stats* st);
int cube_pm_coarse_density(cube_ctx* ctx, cube_stats* st);
int cube_pm_fine_forces(cube_ctx* ctx, cube_stats* st);
int cube_pm_fine_kick(cube_ctx* ctx, float a_mid, float dt);
int cube_pm_coarse_forces(cube_ctx* ctx, cube_stats* st);
int cube_pm_coarse_kick(cube_ctx* ctx, float a_mid, float dt, cube_stats* st);

/* Power spectrum of the resident particles (cicpower.f90 + powerspectrum.f90
   cross_power): CIC density on an ng^3 mesh (ng = nc, 2 nc or 4 nc; mass 1,
   position (cell+frac)*ng/nc - 0.5), density contrast, R2C, linear bins
   ibin = nint(|k|) for ibin = 1..nbin with nbin >= cube_pk_nbin(ng) =
   nint(ng/2*sqrt(3)).  delta2: optional second density contrast (host,
   ng^3 float, Fortran order) for the cross power; NULL gives the auto power.
   xi receives xi(10, nbin) in the reference's meaning: modes, k (h/Mpc, box
   in Mpc/h), Delta^2_11, Delta^2_22, Delta^2_12, <1/sinc^2>, <1/sinc^4>, r,
   b, reconstructed power.  Uses the fine-mesh buffers as scratch. */
int cube_pk_nbin(int ng);
int cube_power_spectrum(cube_ctx* ctx, int ng, float box, const float* delta2, double* xi, int nbin);

int cube_get_field(cube_ctx* ctx, int field, void* host);
int cube_set_field(cube_ctx* ctx, int field, const void* host);

/* Number of particles currently resident. */
int64_t cube_nplocal(const cube_ctx* ctx);
int cube_synchronize(cube_ctx* ctx);

/* Per-phase device timers (replace the reference's system_clock prints,
   e.g. pm.f90:35-411): enable=1 resets and starts event pairs around every
   phase on the context's stream, enable=0 stops; cube_timing_read harvests
   the accumulated milliseconds and launch counts per phase. */
#define CUBE_NPHASE 16
int cube_timing(cube_ctx* ctx, int enable);
int cube_timing_read(cube_ctx* ctx, double* ms, int64_t* count, int nphase);
const char* cube_phase_name(int phase);
/* The CUDA stream (cudaStream_t) all of the context's work is issued on. */
void* cube_stream(cube_ctx* ctx);

/* Run-time options.  CUBE_OPT_EXACT_KICKS=1 makes every kernel evaluate the
   reference's FP64 expressions directly instead of the certified FP32 /
   float-float fast paths (results are identical by construction; used to test
   that claim and to time it).  CUBE_OPT_PP_LEVEL=2 sets the first of the
   six PP levels (0: 4^3-cell bricks staged in shared memory, the default;
   1: bricks in a large block; 2: single cells; 3: single cells in a large
   block; 4: single cells staged in a global scratch, a region per block;
   5: the same with the whole scratch), which otherwise serve only regions
   too dense for the level before.  Every level sums a particle's pairs in
   the same order, so every level gives bitwise the same result; used to
   test the dense-region paths.  CUBE_OPT_RANK_WALK=3 picks how
   cube_update_x finds each particle's rank in its destination cell (the
   reference's visit order): 0 (default) the counting path when every
   particle moved at most one cell and landed in one frame, else a radix
   sort on (destination, place of the source cell in the destination's visit
   order, index in the source cell); 1 the visit-order walker (one thread per
   destination walking its source cells); 2 the sort always.  Same result
   for all.
   CUBE_OPT_DEPOSIT_FINE=4 / CUBE_OPT_DEPOSIT_COARSE=5 pick the brick shape
   of the fine / coarse density deposit (0-3; fine: 8x4x4, 4x4x4, 8x4x2,
   4x4x2 coarse cells; coarse: 8x8x8, 16x8x8, 8x8x4, 4x4x4): a tile-size
   choice for the autotuner, same exact sums for every shape.
   CUBE_OPT_FAIL_ALLOC=6 is host-side fault injection for tests: value n > 0
   makes the n-th device allocation the library makes lazily (the general
   re-sort's key buffers, on first use) report failure, 0 turns it off.
   CUBE_OPT_PP_HEAVY=7 sets how many neighbour entries make a particle of a
   crowded PP block walked by a whole warp instead of one thread (0: the
   default, 8192); the two walks give bitwise the same sums, so this too only
   serves tests and timing.  CUBE_OPT_PP_PARTS=8 caps the parts a dense PP
   brick or cell is split into, each part on its own SM (0: the default cap,
   255; 1: no split); same sums for every value.  CUBE_OPT_PP_FILTER=9
   controls PP's prefilter: a particle whose 27 neighbouring fine cells hold
   no other particle gets a zero pair force (its list is the one entry of
   itself, as in the reference's loop), found from per-cell occupancy masks,
   and the staging levels then see only the other particles, whose lists are
   unchanged.  0 (default): on while the last filtered call found fewer than
   half the particles with a neighbour, re-tried every 16th call otherwise,
   and always inside the batched ensemble's captured graphs; 1: off; 2: on.
   Bitwise the same forces, pair counts and codes. */
enum cube_option {
  CUBE_OPT_EXACT_KICKS = 1,
  CUBE_OPT_PP_LEVEL = 2,
  CUBE_OPT_RANK_WALK = 3,
  CUBE_OPT_DEPOSIT_FINE = 4,
  CUBE_OPT_DEPOSIT_COARSE = 5,
  CUBE_OPT_FAIL_ALLOC = 6,
  CUBE_OPT_PP_HEAVY = 7,
  CUBE_OPT_PP_PARTS = 8,
  CUBE_OPT_PP_FILTER = 9
};
int cube_set_option(cube_ctx* ctx, int option, int64_t value);

/* Velocity-code self check: encodes n host doubles with sigma both by the
   direct FP64 formula of update_particle.f90:117 and by the table path the
   kernels use; writes both codes (host arrays of n int32). */
int cube_codec_check(cube_ctx* ctx, float sigma, const double* v, int64_t n, int32_t* direct, int32_t* table);

/* Arithmetic self check: the kick terms divide by 6 and by pi_f with an
   FMA-corrected reciprocal product instead of the IEEE division; this runs
   both over every float bit pattern (NaN excluded) and writes the number of
   differing results for each divisor into mismatches[0..1] (expected 0). */
int cube_arith_check(cube_ctx* ctx, int64_t* mismatches);

/* cube_codec_check without any device allocation (no counterpart in the
   reference): all of its device scratch -- CUBE_CODEC_STATIC_MAX input
   values, their two outputs and one set of codec tables (1.5 MiB in all) --
   is a fixed file-scope array that every GPU loading the library holds until
   exit.  It is for callers that must not allocate: a run whose particle
   arrays fill HBM (a mid-run cudaMalloc can fail there), or a monitor that
   must not trigger cudaFree's device-wide synchronisation.  n >
   CUBE_CODEC_STATIC_MAX returns CUBE_ERR_ARG.  The call builds its own codec
   tables for sigma in the array, so the context's tables for the step's
   sigma_vi / sigma_vi_new stay as they were.  The first call on each device
   resolves the array's address and should come before any stream capture.
   Calls on one device share the array and are serialised by a host lock that
   covers only that array; each returns after the context's stream has
   drained.  The call runs on the context's stream, so a monitoring thread
   uses a context of its own (calls on one context must not overlap). */
#define CUBE_CODEC_STATIC_MAX 16384
int cube_codec_check_static(cube_ctx* ctx, float sigma, const double* v, int64_t n, int32_t* direct,
                            int32_t* table);

/* ------------------------------------------------------------------------
   Batched ensemble (no reference counterpart: the reference runs one
   universe per job and batches jobs with shell scripts).  Independent boxes,
   each a single-tile image with its own sizes, cosmology and seed (Zel'dovich
   initial conditions of cube_ic_zeldovich) and its own fixed step schedule.
   CUBE_BATCH_GRAPH advances every box one step per launch of a captured CUDA
   graph (one branch per box, the plain path's kernels, every per-step
   decision on the device); CUBE_BATCH_SERIAL runs the same schedule through
   the plain entry points one box after another.  Both give the same state. */
typedef struct cube_batch cube_batch;
typedef struct cube_batch_box {
  cube_params params;    /* nnt = 1 */
  cube_cosmology cosmo;
  float z_init;
  uint32_t seed;
} cube_batch_box;
typedef struct cube_batch_stats {  /* one box, one step */
  float sigma_vi_new;
  float f2_max_fine, f2_max_coarse, f2_max_pp;
  float vmax[3];
  int32_t flags;       /* update_x flags: 1 displacement, 2 rank, 4/8 walker used */
  int64_t npairs, itest1, ndup;
  double sum_r;        /* sigma sum of squares */
} cube_batch_stats;
#define CUBE_BATCH_GRAPH 0
#define CUBE_BATCH_SERIAL 1
int cube_batch_create(const cube_batch_box* boxes, int nbox, const float* fine_table, const float* coarse_table,
                      int device, int mode, cube_batch** out);
int cube_batch_destroy(cube_batch* batch);
const char* cube_batch_last_error(const cube_batch* batch);
/* dt and a_mid per box and step, host arrays [nbox][nsteps]; dt_old of the
   first step is 0 (timestep.f90:4) */
int cube_batch_set_schedule(cube_batch* batch, int nsteps, const float* dt, const float* a_mid);
/* per distinct box geometry, by device time on the box's initial state: the
   fine and coarse deposits' brick shapes (CUBE_OPT_DEPOSIT_FINE / _COARSE)
   and the PP start level (which staging tiles carry the pairs); choices
   (3 x nbox int32, may be null) receives (PP level, fine shape, coarse
   shape) per box.  Results do not depend on the choices. */
int cube_batch_autotune(cube_batch* batch, int32_t* choices);
/* advance every box nsteps steps of its schedule */
int cube_batch_step(cube_batch* batch, int nsteps);
int cube_batch_history(cube_batch* batch, int step, cube_batch_stats* out);  /* nbox entries */
int cube_batch_ctx(cube_batch* batch, int box, cube_ctx** ctx);  /* the box's context */
int cube_batch_time(const cube_batch* batch, float* last_ms, float* last_dev_ms, int64_t* steps_done);
/* per step done so far, the time of that step over all boxes (ms; device
   time between graph launches, or the serial wall clock summed over boxes) */
int cube_batch_step_times(const cube_batch* batch, float* ms);

/* ------------------------------------------------------------------------
   Differentiable form (no reference counterpart: the reference has no
   gradients).  A single-level PM integrator on decoded FP32 positions --
   deposit, Green's multiply (-4 pi/khat^2), central-difference force, kick,
   drift with the coefficients of the reference's step (drift = dt_mid of
   update_particle.f90:66, kick = a_mid*dt/(6 pi) of pm.f90:162) -- from
   Zel'dovich initial conditions of white noise on the npd^3 particle lattice
   (the filter of cube_ic_zeldovich), with hand-written adjoint kernels.
   Positions are displacements d from each particle's lattice point (the
   centre of mesh cell step*l, step = ng/npd) in mesh cells, unwrapped;
   particles in lattice order l = x + npd*(y + npd*z); arrays (3, np) float.  Every pointer of the pass calls is
   DEVICE memory on the context's device; the calls return after the
   context's stream has drained.  cube_dpm_backward applies to the last
   cube_dpm_forward (its checkpoints); the state is kept at the start of
   every ckpt_every steps and the rest recomputed. */
typedef struct cube_dpm cube_dpm;
typedef struct cube_dpm_params {
  int32_t ng;          /* mesh cells per dimension (even, >= 16) */
  int32_t npd;         /* particles and noise points per dimension (even, >= 16, divides ng) */
  int32_t max_steps;   /* schedule capacity */
  int32_t ckpt_every;  /* steps per recomputation segment (1 keeps every step) */
  float z_init;        /* redshift of the initial conditions */
} cube_dpm_params;

int cube_dpm_create(const cube_dpm_params* params, const cube_cosmology* cosmo, int device, cube_dpm** out);
int cube_dpm_destroy(cube_dpm* ctx);
const char* cube_dpm_last_error(const cube_dpm* ctx);
void* cube_dpm_stream(cube_dpm* ctx);
int64_t cube_dpm_nparticles(const cube_dpm* ctx);
/* per-step drift (dt_mid) and kick (a_mid*dt/(6 pi)) coefficients, host arrays */
int cube_dpm_set_schedule(cube_dpm* ctx, int nsteps, const float* drift, const float* kick);
/* npd^3 Gaussian white noise of a seed (the generator of cube_ic_zeldovich) */
int cube_dpm_noise(cube_dpm* ctx, uint32_t seed, float* noise);
/* noise (npd^3) -> final displacements and velocities (3, np) */
int cube_dpm_forward(cube_dpm* ctx, const float* noise, float* x, float* v);
/* cotangents of the final (x, v) -> of the noise; gx0 / gv0 (optional)
   receive those of the initial state */
int cube_dpm_backward(cube_dpm* ctx, const float* gx, const float* gv, float* gnoise, float* gx0, float* gv0);
/* CIC density (ng^3, mean 1) of displacements x, and its adjoint gx = (d rho/d x)^T grho */
int cube_dpm_density(cube_dpm* ctx, const float* x, float* rho);
int cube_dpm_density_adjoint(cube_dpm* ctx, const float* x, const float* grho, float* gx);
/* HOST copies of the IC filter ((npd/2+1) npd^2) and Green's function
   ((ng/2+1) ng^2), both with the inverse transform's 1/n^3 folded in */
int cube_dpm_tables(cube_dpm* ctx, float* ic_filter, float* green);
/* particle mass, a^2 H at z_init, and the device times of the last forward
   and backward pass (CUDA events around each graph launch) */
int cube_dpm_info(const cube_dpm* ctx, float* mass, float* vf, float* fwd_ms, float* bwd_ms);

#ifdef __cplusplus
}
#endif
#endif /* CUBE_GPU_H */
