/*
 * kestrel_gpu.h -- C ABI of the GB300 implementation of Kestrel's time-step hot path.
 *
 * The reference (Kestrel v1.1.1, serial Fortran 2008) has no plugin interface for its
 * hot path: the module procedures below are called directly from `Run`
 * (src/TimeStepper.f90:73) and `main` (src/main.f90:171).  This header is the drop-in
 * boundary a Fortran host binds with ISO_C_BINDING, in the same way the reference already
 * binds its C++ glue (src/GeoTiffRead.f90:43-100 <-> src/RasterData.h:181-,
 * src/version.f90:25-33 <-> src/cversion.cpp:28-34): one interface block per entry point,
 * bind(C, name="kg_...") with value arguments for scalars and handles.
 *
 * Conventions
 *  - Every entry point returns an int status: 0 (KG_OK) or a negative KG_ERR_* code.  The
 *    library never calls exit/abort and never traps on the device.  kg_last_error() gives
 *    a one-line message for the last failure on a context; kg_last_error(NULL) gives the
 *    reason the calling thread's last kg_create failed.
 *  - All pointers in signatures are HOST pointers; the context owns every device buffer.
 *  - Indices are 1-based tile IDs exactly as in the reference (src/Grid.f90:260-267,
 *    id = i + (j-1)*nXtiles, tiles numbered from the south-west corner).
 *  - Per-tile cell arrays are nXpertile*nYpertile doubles, i (x) fastest, i.e. the
 *    reference's u(d, :, :) slice for one field d (src/Grid.f90:83).
 *  - One context = one simulation on one GPU and one CUDA stream; calls on the same
 *    context are not thread-safe, separate contexts are independent.
 */
#ifndef KESTREL_GPU_H
#define KESTREL_GPU_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* ---- status codes (replace FatalErrorMessage / exit(1), src/Messages.f90:56-90) ---- */
#define KG_OK                 0
#define KG_ERR_PARAM         -1  /* invalid parameter value (src/Parameters.f90 FatalError_*) */
#define KG_ERR_OOM           -2  /* device memory (cudaErrorMemoryAllocation) or host memory ran out */
#define KG_ERR_HALT_EDGE     -3  /* flow reached the domain edge under 'halt' (src/UpdateTiles.f90:61-69) */
#define KG_ERR_NAN           -4  /* reserved: like the reference, a step does not scan the state for
                                     non-finite values; a non-finite advised dt gives KG_ERR_DT */
#define KG_ERR_CUDA          -5  /* CUDA runtime error */
#define KG_ERR_UNSUPPORTED   -6  /* configuration outside the implemented path (e.g. 1D grids) */
#define KG_ERR_STATE         -7  /* call out of order (e.g. stepping before sources are loaded) */
#define KG_ERR_DT            -8  /* time step collapsed: dt <= 0 or not finite, or 100000
                                     refinements of one step (the reference would loop on) */
#define KG_ERR_NOT_FOUND     -9  /* requested tile is not active */
#define KG_ERR_TIMEOUT      -10  /* reserved: no kernel of the library waits on a flag */

/* ---- runtime closure selections (procedure pointers in the reference) ---- */
/* Drag: src/Parameters.f90:222-247, src/Closures.f90:365-558 */
enum { KG_DRAG_CHEZY = 0, KG_DRAG_COULOMB = 1, KG_DRAG_VOELLMY = 2, KG_DRAG_POULIQUEN = 3,
       KG_DRAG_EDWARDS2019 = 4, KG_DRAG_VARIABLE = 5, KG_DRAG_MANNING = 6 };
/* Erosion: src/Parameters.f90:285-310, src/Closures.f90:566-675 */
enum { KG_ERO_OFF = 0, KG_ERO_MIXED = 1, KG_ERO_SIMPLE = 2, KG_ERO_FLUID = 3, KG_ERO_GRANULAR = 4 };
/* Deposition: src/Parameters.f90:163-176, src/Closures.f90:320-356 */
enum { KG_DEP_NONE = 0, KG_DEP_SIMPLE = 1, KG_DEP_SPEARMAN_MANNING = 2 };
/* Erosion transition: src/Closures.f90:684-732 */
enum { KG_ETRANS_SMOOTH = 0, KG_ETRANS_STEP = 1, KG_ETRANS_OFF = 2 };
/* Morphodynamic damping: src/Closures.f90:744-791 */
enum { KG_DAMP_NONE = 0, KG_DAMP_TANH = 1, KG_DAMP_RAT3 = 2 };
/* Switch function: src/Closures.f90:797-915 */
enum { KG_SWITCH_TANH = 0, KG_SWITCH_RAT3 = 1, KG_SWITCH_COS = 2, KG_SWITCH_LINEAR = 3,
       KG_SWITCH_EQUAL = 4, KG_SWITCH_ZERO = 5, KG_SWITCH_ONE = 6, KG_SWITCH_STEP = 7 };
/* Slope limiter: src/SolverSettings.f90:102-126, src/Limiters.f90:83-184 */
enum { KG_LIM_MINMOD1 = 0, KG_LIM_MINMOD2 = 1, KG_LIM_VANALBADA = 2, KG_LIM_WENO = 3, KG_LIM_NONE = 4 };
/* Boundary conditions: src/DomainSettings.f90:108-120 */
enum { KG_BC_HALT = 0, KG_BC_PERIODIC = 1, KG_BC_DIRICHLET = 2, KG_BC_SPONGE = 3 };
/* Analytic topography (src/TopogFuncs.f90) or an uploaded vertex grid (kg_upload_b0). */
enum { KG_TOPO_UPLOAD = 0, KG_TOPO_FLAT = 1, KG_TOPO_XSLOPE = 2, KG_TOPO_YSLOPE = 3,
       KG_TOPO_XYSLOPE = 4, KG_TOPO_XSINSLOPE = 5, KG_TOPO_XYSINSLOPE = 6, KG_TOPO_XHUMP = 7,
       KG_TOPO_XTANH = 8, KG_TOPO_XPARAB = 9, KG_TOPO_XYPARAB = 10,
       KG_TOPO_RASTER = 11 /* a georeferenced elevation raster (kg_upload_raster) */,
       KG_TOPO_X2SLOPES = 12, KG_TOPO_USGS = 13, KG_TOPO_FLUME = 14, KG_TOPO_CHANNEL_POWERLAW = 15,
       KG_TOPO_CHANNEL_TRAPEZIUM = 16, KG_TOPO_XBISLOPE = 17, KG_TOPO_XTRISLOPE = 18 };
/* Cap / cube shapes: src/InitConds.f90:499-510, :705-712 */
enum { KG_SHAPE_FLAT = 0, KG_SHAPE_PARA = 1, KG_SHAPE_LEVEL = 2 };
/* Arithmetic form of the GPU path. */
enum { KG_PREC_FP64 = 0, KG_PREC_FP32 = 1 };

#define KG_MAX_CAPS     16
#define KG_MAX_CUBES    16
#define KG_MAX_SOURCES  16
#define KG_MAX_SERIES   64
#define KG_MAX_TOPO_PARAMS 8

typedef struct {                       /* src/InitConds.f90 type Caps */
    double x, y, radius, height, psi, u, v;
    int32_t shape, _pad;
} kg_cap;

typedef struct {                       /* src/InitConds.f90 type Cubes */
    double x, y, length, width, height, psi, u, v;
    int32_t shape, _pad;
} kg_cube;

typedef struct {                       /* src/InitConds.f90 type Sources */
    double x, y, radius;
    int32_t n_series, _pad;
    double time[KG_MAX_SERIES];
    double flux[KG_MAX_SERIES];
    double psi[KG_MAX_SERIES];
} kg_flux_source;

/*
 * Every numeric RunSet field the hot path reads (src/RunSettings.f90:161-340), with the
 * reference's defaults applied by the host-side parser (kestrel_gb300/config.py).  The
 * derived quantities (gred, Rep, ws0, nsettling, CriticalShields, diffusiveTimeScale,
 * deltaX/Y; src/Parameters.f90:629-648, src/DomainSettings.f90:196-225) are computed by
 * kg_create from these.
 */
typedef struct {
    /* Domain block */
    int32_t nXtiles, nYtiles, nXpertile, nYpertile;
    double  Xtilesize, Ytilesize;
    int32_t bcs, _pad0;
    double  bcsHnval, bcsuval, bcsvval, bcspsival;
    /* Parameters block */
    int32_t geometric_factors, MorphodynamicsOn;
    double  g, rhow, rhos;
    double  ChezyCo, ManningCo, CoulombCo;
    double  PouliquenMinSlope, PouliquenMaxSlope, PouliquenIntermediateSlope, PouliquenBeta;
    double  Edwards2019betastar, Edwards2019kappa, Edwards2019Gamma;
    double  VoellmySwitchRate, VoellmySwitchValue;
    double  EroRate, EroRateGranular, EroDepth, EroCriticalHeight, BedPorosity;
    double  maxPack, SolidDiameter, EddyViscosity;
    int32_t ws0_given, _pad1;           /* 'Settling speed' key overrides the derived ws0 */
    double  ws0;
    int32_t drag, erosion, deposition, erosion_transition, morpho_damping, fswitch;
    /* Solver block */
    int32_t limiter, TileBuffer;
    double  heightThreshold, cfl, maxdt, tstart, tend, SpongeStrength;
    /* Output block: Nout fixes the IntegrateTo end points (src/TimeStepper.f90:97-103) */
    int32_t Nout, _pad2;
    /* Initial conditions */
    int32_t nCaps, nCubes, nSources, _pad3;
    kg_cap  caps[KG_MAX_CAPS];
    kg_cube cubes[KG_MAX_CUBES];
    kg_flux_source sources[KG_MAX_SOURCES];
    /* Topog block */
    int32_t topog, n_topog_params;
    double  topog_params[KG_MAX_TOPO_PARAMS];
} kg_params;

/* Per-call statistics of kg_step / kg_integrate_to. */
typedef struct {
    double  t;                  /* simulation time after the call */
    double  dt;                 /* last accepted hydraulic dt (dt_hydro) */
    int64_t steps;              /* accepted steps taken by this call */
    int64_t rejected;           /* dt refinements (rejected attempts) in this call */
    int64_t cell_updates;       /* active cells x accepted hydraulic steps (H.M.H counts 2) */
    int32_t n_active, n_ghost;  /* tile counts after the call */
    int64_t kernel_launches;    /* device kernels launched by this call */
} kg_step_stats;

typedef struct kg_ctx kg_ctx;

/* Library version string (src/version.f90 GetVersion analogue). */
const char* kg_version(void);

/* InitialiseGrid (src/Grid.f90:166) + topography set-up (src/dem.f90 LoadDEM). precision
   selects the FP64 drop-in (KG_PREC_FP64) or the FP32 mixed form (KG_PREC_FP32).
   The struct is checked before the device is touched: tile counts and sizes, positive cfl,
   heightThreshold and maxdt, counts of caps/cubes/sources and series lengths, and every
   selector within its enum give KG_ERR_PARAM (a 1D grid KG_ERR_UNSUPPORTED); then no
   device gives KG_ERR_CUDA.  On failure *out is NULL and kg_last_error(NULL) says why. */
int  kg_create(const kg_params* params, int32_t precision, kg_ctx** out);
void kg_destroy(kg_ctx* ctx);
const char* kg_last_error(const kg_ctx* ctx);

/* Replaces GetTileHeights (src/dem.f90:395-416) with a global vertex grid of
   (nXtiles*nXpertile+1) x (nYtiles*nYpertile+1) heights, x fastest, vertex (0,0) at the
   south-west domain corner.  Must be called before kg_load_sources when topog==UPLOAD. */
int  kg_upload_b0(kg_ctx* ctx, const double* b0_vertices, int64_t nx1, int64_t ny1);

/* Georeferencing of an elevation raster, as GDAL reports it for the reference's DEM.vrt
   (src/RasterData.cpp:160-215): the geotransform's origin and pixel sizes (north-up:
   pixel_w > 0, pixel_h < 0), the no-data value, and the projected coordinates of the
   domain centre (RunParams%centerUTM, src/TopogSettings.f90:387). */
typedef struct {
    int64_t nx, ny;              /* RasterXSize, RasterYSize */
    double origin_x, origin_y;   /* geotransform[0], geotransform[3]: upper-left corner */
    double pixel_w, pixel_h;     /* geotransform[1], geotransform[5] */
    double nodata;
    double center_e, center_n;
} kg_raster;

/* Replaces the raster branch of GetTileHeights (TileHeightData and GetRasterData,
   src/dem.f90:203-356, with Bicubic_r, src/Interp2d.f90:214-282): values are the raster's
   ny x nx elevations, row 0 the top (north) row, x fastest (GDAL RasterIO order).  Each
   tile's vertex heights are the mean of four bicubic samples at the vertex's surrounding
   cell corners, taken from the tile's own raster section exactly as the reference takes
   them; a tile whose section leaves the raster or holds the no-data value fails with
   KG_ERR_PARAM when it is activated (the reference's fatal read errors,
   src/GeoTiffRead.f90:213-214).  The heights of every tile are computed on the GPU at this
   call.  Must be called before kg_load_sources when topog==RASTER. */
int  kg_upload_raster(kg_ctx* ctx, const double* values, const kg_raster* geo);

/* LoadSourceConditions (src/SetSources.f90:47-405): places caps, cubes and flux sources
   and activates (AddTile) every tile that covers them. */
int  kg_load_sources(kg_ctx* ctx);
/* Restart from a saved state instead of loading the sources (LoadInitialCondition,
   src/Restart.f90:55-328): activates tiles ids[0..n) (strictly increasing) in order and
   sets, per tile k, the conserved fields state[k][4][nYpertile][nXpertile] (w, rhoHnu,
   rhoHnv, Hnpsi) and, when bt_vertex is not NULL, the vertex bed change
   bt_vertex[k][nYpertile+1][nXpertile+1]; the cell and interfacial topography, the ghost
   tiles and the flux-source cell counts are rebuilt; the clock is set to t.  Use on a
   context with nothing loaded (no kg_load_sources). */
int  kg_load_state(kg_ctx* ctx, const int32_t* ids, int32_t n, const double* state, const double* bt_vertex, double t);

/* One accepted time step of IntegrateTo's loop (src/TimeStepper.f90:151-275), ending no
   later than t_stop. */
int  kg_step(kg_ctx* ctx, double t_stop, kg_step_stats* stats);

/* IntegrateTo (src/TimeStepper.f90:116-277): step until t >= t_end. */
int  kg_integrate_to(kg_ctx* ctx, double t_end, kg_step_stats* stats);

/* Run (src/TimeStepper.f90:73-112) without the file output: integrate to each of the Nout
   output times tstart + i*DeltaT in turn. */
int  kg_run(kg_ctx* ctx, kg_step_stats* stats);

/* CalculateHydraulicRHS (src/HydraulicRHS.f90:64-136) applied to the current solution
   (the reference's tileContainer) at time t for the given substep (1..4).  Writes the
   advised time step; the RHS itself is readable with kg_get_tile_rhs. */
int  kg_hydraulic_rhs(kg_ctx* ctx, double t, int32_t substep, double* advised_dt);

/* Sorted active tile list (src/Grid.f90:123 activeTiles%List) and ghost list (append
   order).  *n is in/out: capacity on entry, count on exit. */
int  kg_get_active_tiles(kg_ctx* ctx, int32_t* ids, int32_t* n);
int  kg_get_ghost_tiles(kg_ctx* ctx, int32_t* ids, int32_t* n);

/* The whole active state in one call, the counterpart of kg_load_state (the state the
   reference's snapshot writers read from grid%tileContainer, src/Output.f90:754-931, and
   its restart reader takes back, src/Restart.f90:55-328): the active tile ids in list
   order, per tile k the conserved fields state[k][4][nYpertile][nXpertile] (w, rhoHnu,
   rhoHnv, Hnpsi) and the vertex bed change bt_vertex[k][nYpertile+1][nXpertile+1].  One
   device gather, one copy per array, one wait.  *n is in/out: capacity on entry, count
   on exit; with ids, state and bt_vertex all NULL only the count is returned.  Any of the
   three may be NULL.  KG_ERR_PARAM when the capacity is below the count. */
int  kg_get_state(kg_ctx* ctx, int32_t* ids, int32_t* n, double* state, double* bt_vertex);

/* One field (1..13, src/main.f90:116-141) of the current solution for an active tile,
   nXpertile*nYpertile doubles.  Fields 5..9 are the desingularised variables as the
   reference holds them in tileContainer after the last step. */
int  kg_get_tile_field(kg_ctx* ctx, int32_t tile_id, int32_t field, double* out);
/* Overwrite one of the conserved fields 1..4 of an active tile (tests, restarts). */
int  kg_set_tile_field(kg_ctx* ctx, int32_t tile_id, int32_t field, const double* in);
/* Vertex bed of an active tile, (nXpertile+1)*(nYpertile+1) doubles: which=0 b0, 1 bt. */
int  kg_get_tile_vertex(kg_ctx* ctx, int32_t tile_id, int32_t which, double* out);
/* ddtExplicit (k=1..4) / ddtImplicit (k=5, momenta) of the last kg_hydraulic_rhs call. */
int  kg_get_tile_rhs(kg_ctx* ctx, int32_t tile_id, int32_t k, double* out);
/* Running maxima (src/TimeStepper.f90:1155-1303): which = 0 Hnmax, 1 umax, 2 emax,
   3 dmax, 4 psimax (value plane then time plane, 2*nX*nY doubles), 5 tfirst (nX*nY). */
int  kg_get_tile_maxima(kg_ctx* ctx, int32_t tile_id, int32_t which, double* out);

/* CalculateVolume (src/Output.f90:617-737): out = {volume, total_bed_volume, total_mass,
   total_solids} before the rho multipliers, i.e. the four Kahan sums times dx*dy. */
int  kg_volume(kg_ctx* ctx, double out[4]);

/* Current time, last dt and the number of device kernels launched so far. */
int  kg_get_time(kg_ctx* ctx, double* t, double* dt);
int64_t kg_kernel_launches(const kg_ctx* ctx);

/* The cudaStream_t the context launches on, so a caller can order (or time) its own work
   against the library's.  No reference counterpart (the reference has no device). */
void* kg_stream(kg_ctx* ctx);
/* When enabled, every fused hydraulic pass is bracketed by CUDA events on the context's
   stream; kg_get_kernel_time returns the accumulated pass duration in ms and the count.
   No reference counterpart. */
int  kg_set_kernel_timing(kg_ctx* ctx, int32_t enable);
int  kg_get_kernel_time(kg_ctx* ctx, double* ms, int64_t* passes);
/* FP32 form: run each stage of the morphodynamic operator (E - D, the vertex source and bed
   update, the cell bed and w / Hnpsi update; MorphodynamicTimeStepper, src/TimeStepper.f90:
   569-699) as one launch (enable, the default) or as three (0); the results are the same bit
   for bit.  No effect on the FP64 form or on batch members (the batched engine runs the
   three launches, with the same results).  No reference counterpart. */
int  kg_set_fused_morpho(kg_ctx* ctx, int32_t enable);
/* FP32 form: skip the reconstruction, flux and RHS work of a 16 x 16 block whose cells and
   two-cell halo hold no water (depth above the bed, Hnpsi and momenta all within
   1e-4 heightThreshold) and no flux source, carrying its state forward with a zero RHS
   (enable, the default), or run every block in full (0).  The difference is round-off of
   the dry bed (face depths of order 1e-13 m).  No effect on the FP64 form, which always
   runs every block as the reference does.  No reference counterpart. */
int  kg_set_dry_skip(kg_ctx* ctx, int32_t enable);
/* Redistribution work so far (RedistributeGrid, src/Redistribute.f90:203-244): the number
   of listed cells walked, the dependency waves they were run in and the walks.  No
   reference counterpart (the reference walks its list serially). */
int  kg_redistribution_stats(kg_ctx* ctx, int64_t* cells, int64_t* waves, int64_t* walks);
/* Accepted steps, refused attempts and cell-updates (active cells x accepted hydraulic
   steps) so far; and the device bytes the context holds for its allocated tiles.  No
   reference counterpart. */
int  kg_get_counters(kg_ctx* ctx, int64_t out[3]);
int64_t kg_device_bytes(kg_ctx* ctx);
/* Device bytes one allocated tile (active or ghost) costs for the given tile size and
   form; host arithmetic only, no device needed (0 for invalid arguments).  A context's
   tile memory is this times its slot capacity. */
int64_t kg_slot_bytes(int32_t nXpertile, int32_t nYpertile, int32_t precision);
/* Bytes copied host->device (out[0]) and device->host (out[1]) by the context so far. */
int  kg_get_transfer_bytes(kg_ctx* ctx, int64_t out[2]);
/* Host wall time in seconds since creation: out[0] inside kg_step/kg_integrate_to steps,
   out[1] of that blocked in stream synchronisations (the host waiting for the GPU),
   out[2] planning redistribution walks.  No reference counterpart. */
int  kg_host_times(kg_ctx* ctx, double out[3]);

/* Same as kg_hydraulic_rhs (substep 1..4, advised dt, ddtExplicit/ddtImplicit readable
   with kg_get_tile_rhs) but allocates nothing: for hosts that own all device memory and do
   not let a library call cudaMalloc once running.  The pass's scratch (its CFL-minimum
   word and tile-block list) lives in one static device array of about 1 MiB that every
   GPU loading the library keeps until exit; at most 65,536 blocks of 16x16 cells (about
   16.7 M active cells) are accepted, more is KG_ERR_PARAM.  All calls share that array, so
   calls that overlap on the GPU race.  The first call on a device looks up the array's
   address (cudaGetSymbolAddress, once per device); make it before any stream capture.
   No counterpart in the reference. */
int  kg_hydraulic_rhs_noalloc(kg_ctx* ctx, double t, int32_t substep, double* advised_dt);

/* ---- Batched ensemble: many FP32-form simulations advanced together ----------------
   The hydraulic passes of all members run as one persistent launch over their packed
   tile blocks; each member keeps its own tiles, dt control and refinement history, so its
   results do not depend on the other members.  No reference counterpart (the reference
   runs one simulation per process). */
typedef struct kg_batch kg_batch;
int  kg_batch_create(int32_t max_members, kg_batch** out);
void kg_batch_destroy(kg_batch* b);
const char* kg_batch_last_error(const kg_batch* b);
/* Add a member from its run settings (always the FP32 form); b0 is the vertex grid for
   KG_TOPO_UPLOAD (else NULL); its sources are loaded.  id receives the member id. */
int  kg_batch_add(kg_batch* b, const kg_params* params, const double* b0, int64_t nx1, int64_t ny1, int32_t* id);
/* The member's context: the single-simulation getters (kg_get_tile_field, kg_volume,
   kg_get_time, ...) work on it.  Do not step or destroy it directly. */
kg_ctx* kg_batch_member(kg_batch* b, int32_t id);
int  kg_batch_remove(kg_batch* b, int32_t id);
/* One round of every member that has not reached its end time: each advances its current
   step (IntegrateTo's, src/TimeStepper.f90:151-275, through its output intervals as
   kg_run takes them) by one phase, at most completing it; members at the same stage share
   the batched launches.  live receives the number of members still running. */
int  kg_batch_step(kg_batch* b, int32_t* live);
int  kg_batch_finished(kg_batch* b, int32_t id, int32_t* finished);
int  kg_batch_stats(kg_batch* b, int64_t* launches, int64_t* rounds);
void* kg_batch_stream(kg_batch* b);
/* CUDA graphs for the rounds (on by default): each device segment of a round between two
   waits -- the batched H phase, the M operator up to its checks, the closing launch with the
   RHS check and second H -- runs as one executable graph per segment kind: launched as it
   is when the segment's launches and copies carry the same parameters as last time (the
   tables they read are refreshed in pinned memory), else captured from the batch stream
   and updated in place, or instantiated when its shape changed.  enable = 0 launches the
   same work directly on the stream. */
int  kg_batch_set_graphs(kg_batch* b, int32_t enable);
/* out[0] graph launches, out[1] in-place updates, out[2] instantiations, out[3] launches
   of an unchanged graph without a capture, so far. */
int  kg_batch_graph_stats(kg_batch* b, int64_t out[4]);

#ifdef __cplusplus
}
#endif
#endif /* KESTREL_GPU_H */
