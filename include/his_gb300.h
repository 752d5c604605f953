/*
 * his_gb300.h -- C ABI of the GB300-native flood-engine time step.
 *
 * Plain C: opaque handles, plain pointers and sizes, int status codes.  Device
 * pointers are CUDA device addresses (e.g. torch tensors' data_ptr()); "host"
 * arrays are ordinary host memory copied by the call.  `stream` is a
 * cudaStream_t passed as void* (0 = legacy default stream).  Every call is
 * asynchronous on `stream` unless it returns host results, in which case it
 * synchronises that stream before returning.
 *
 * Each entry point cites the reference interface it replaces (file:line in the
 * reference project hydrointel, Elciiid/HIS).
 */
#ifndef HIS_GB300_H
#define HIS_GB300_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* ---------------------------------------------------------------- status codes */
#define HIS_OK 0
#define HIS_ERR_BAD_ARG 1        /* shape/count mismatch, bad kind, null pointer -> Python ValueError   */
#define HIS_ERR_NONFINITE 2      /* a member's state went non-finite -> NumericalInstabilityError       */
#define HIS_ERR_IMPLAUSIBLE 3    /* a member's state is physically impossible -> NumericalInstabilityError */
#define HIS_ERR_WAIT_TIMEOUT 4   /* a bounded device wait gave up                                        */
#define HIS_ERR_OOM_ADMISSION 5  /* request does not fit the HBM budget                                  */
#define HIS_ERR_CUDA 6           /* CUDA runtime error (message via his_last_error)                      */
#define HIS_ERR_UNSUPPORTED 7    /* feature not available in this library                                */

#define HIS_PREC_F64 0           /* plain method: all arithmetic float64                                  */
#define HIS_PREC_F32 1           /* production form: float32 state and fluxes, float64 accumulators      */

/* Edge order of bc[] and boundary values: west, east, south, north (row 0 = south).
 * Kinds: 0 closed, 1 transmissive, 2 stage, 3 discharge.
 * Replaces: hydrointel/solver/boundaries.py:25-46 (EDGES, EdgeBC, edge_values). */

/* Solver constants.  Replaces hydrointel/config.py:96-131 (SolverConfig). */
typedef struct his_solver_cfg {
    double g, h_dry, kp_eps, cfl, dt_min, dt_max;
    double cfl_1d, slot_width_frac, weir_cw, exchange_limit, exchange_relax;
    int32_t order;   /* 1 or 2 (MUSCL + SSP-RK2) */
    int32_t hllc;    /* 1 HLLC, 0 HLL */
} his_solver_cfg;

/* One member of a 2-D grid set: its own grid size, spacing, edges and fields.
 * All pointers are device pointers of the set's precision (double* or float*),
 * row-major (ny, nx).  Fields may alias between members (a shared bed).
 * storage, f0/fc/k and rain_weight may be NULL (feature off).
 * Replaces the state and fields of hydrointel/solver/swe2d.py:114-146 (SWE2D.__init__). */
typedef struct his_grid_desc {
    int32_t ny, nx;
    int32_t bc[4];
    double dx, dy;
    double horton_t0;
    void *h, *hu, *hv, *s_filled, *infil_cum;
    const void *z, *manning, *storage, *f0, *fc, *k, *rain_weight;
    /* optional running maxima over every step (NULL = off): surface depth and speed
     * (replaces the peak fields built from snapshots, hydrointel/api.py:238-241) */
    void *peak_h, *peak_speed;
} his_grid_desc;

/* Per-member forcing of one step: dt, step-start time, rain rate (m/s) and edge
 * values at t and t+dt.  Replaces the packed per-member step quantities of
 * hydrointel/solver/swe2d.py:282-303 (SWE2D._pack / step). */
typedef struct his_step_params {
    double dt, t, rain;
    double bc_t[4], bc_t_dt[4];
} his_step_params;

typedef struct his_grid his_grid;
typedef struct his_net his_net;
typedef struct his_links his_links;

/* Library version and the message of the last failing call on this thread. */
int32_t his_version(void);
const char* his_last_error(void);

/* Create a set of n_members 2-D grids computed in `precision`.  The stencil kernels
 * march up strips of at most tile_x columns (1..346) in chunks of tile_y rows
 * (0, 0 = defaults 58 x 48); the set allocates its own stage scratch.
 * Replaces hydrointel/solver/swe2d.py:113-146 (SWE2D constructor, batched form). */
int32_t his_grid_create(int32_t precision, const his_solver_cfg* cfg, int32_t n_members, const his_grid_desc* grids,
                        int32_t tile_x, int32_t tile_y, his_grid** out);
int32_t his_grid_destroy(his_grid* grid);

/* Bytes of device scratch the set allocated (stage buffers, partials, tables). */
int64_t his_grid_scratch_bytes(const his_grid* grid);

/* Advance every member by one SSP-RK2 step with its own params (host array of
 * n_members).  If vols is non-NULL it receives n_members x 5 float64 volumes
 * (bnd_in, bnd_out, rain, infil, clip; m^3) and the call synchronises `stream`.
 * Large sets run their stage launches as up to 8 parts of whole members on library
 * streams forked from `stream` and joined back into it before the step's totals
 * (his_engine_default_chains' rule), so the parts fill each other's waves; results
 * do not depend on it.
 * Replaces hydrointel/solver/swe2d.py:298-371 (SWE2D.step / _step_core). */
int32_t his_grid_step(his_grid* grid, const his_step_params* params, double* vols, void* stream);

/* Per-member CFL rate max over wet cells of (|u|+c)/dx + (|v|+c)/dy (host out,
 * n_members values; synchronises).  Replaces hydrointel/solver/swe2d.py:179-193
 * (SWE2D._max_rate / max_dt, which reduces over the batch as well). */
int32_t his_grid_max_rate(his_grid* grid, double* rate, void* stream);

/* Asynchronous forms.  They enqueue the same work on `stream` and return without
 * waiting for the GPU: host inputs are copied through pinned staging slots owned by
 * the handle (the caller's arrays may be reused at once), and outputs go to device
 * memory or page-locked host memory (anything else is HIS_ERR_BAD_ARG), valid once
 * `stream` has reached the call.  This is how the reference's step keeps its volumes
 * and mass-balance accumulators on the device (hydrointel/solver/massbalance.py:1-7):
 * a coupled step then waits on the GPU once, for its CFL rates.
 *
 * his_grid_step_async: as his_grid_step; vols (n_members x 5) may be NULL.
 * Replaces hydrointel/solver/swe2d.py:298-371 (SWE2D.step), whose StepVolumes are
 * device tensors. */
int32_t his_grid_step_async(his_grid* grid, const his_step_params* params, double* vols, void* stream);

/* One 2-D step of every member (his_grid_step_async's arguments and asynchrony) that
 * adds its volume terms into a caller's DEVICE ledger instead of returning them:
 * float64, 8 x n_members, row-major, rows rain, infiltration, 2-D boundary in, 2-D
 * boundary out, 1-D boundary in, 1-D boundary out, 2-D clip, 1-D clip (this call adds
 * to rows 0-3 and 6, from the step's own finalize kernel: no extra launch, no copy).
 * Replaces the per-step MassBalance.add of rain, infil, bnd2d_in, bnd2d_out and clip
 * after SWE2D.step (hydrointel/solver/coupling.py:213-218).
 * The first call for a ledger captures the step's kernel launches as a CUDA graph on a
 * library stream; later calls upload the parameters and launch that graph on `stream`
 * (the same kernels and results).  On a stream that is capturing the caller's own
 * graph the launches are issued one by one. */
int32_t his_grid_step_ledger_async(his_grid* grid, const his_step_params* params, double* ledger, void* stream);

/* his_grid_max_rate_async: as his_grid_max_rate into `rate` (n_members).
 * Replaces the reduction of hydrointel/solver/swe2d.py:179-193. */
int32_t his_grid_max_rate_async(his_grid* grid, double* rate, void* stream);

/* The per-member CFL rate of the state the last step left, into `rate` (n_members,
 * device or page-locked memory), without a reduction: the step's last stage forms
 * each cell's rate from the values it stores (the same expression as the reduction)
 * and its finalize keeps the maximum.  Valid only while the state is the last step's
 * output: the caller tracks writes in between (then his_grid_max_rate_async).
 * Replaces the reduction of hydrointel/solver/swe2d.py:179-193 at the start of a
 * coupled step (coupling.py:205-207). */
int32_t his_grid_step_rate_async(his_grid* grid, double* rate, void* stream);

/* Per-member surface and retained volumes sum(h)*area, sum(s_filled)*area (host out,
 * n_members x 2; synchronises).  Replaces hydrointel/solver/swe2d.py:169-174. */
int32_t his_grid_volumes(his_grid* grid, double* vols, void* stream);

/* Bytes of the device scratch compiled into the library for his_grid_step_noalloc
 * (per GPU, held for the life of the process): room for one float64 grid of about
 * 690,000 cells or one float32 grid of about 1,390,000 cells. */
#define HIS_NOALLOC_SCRATCH_BYTES (16u * 1024u * 1024u)

/* One SSP-RK2 step of ONE 2-D grid that allocates no device memory, for callers that
 * may not allocate (an embedding whose host application owns every device allocation,
 * or a one-off step without creating a grid set).  The grid's arrays are described as
 * for his_grid_create, in `precision`; params is one step's forcing; the stage buffers,
 * partial sums and tables live in a fixed library array of HIS_NOALLOC_SCRATCH_BYTES
 * bytes.  Same kernels, decomposition and results as a one-member grid set created
 * with default tiles.  Grids too large for the array return HIS_ERR_BAD_ARG.  The first
 * call in each CUDA context (the device's primary context, or one the application made
 * current itself; a context made after cudaDeviceReset counts as new) looks up the
 * array's address in that context and should come before any stream capture.  Calls
 * share the array: calls that may overlap on the GPU
 * (two streams, two threads) race on it; order them on one stream.  If vols is
 * non-NULL it receives the 5 float64 volumes of his_grid_step and the call
 * synchronises `stream`.
 * No counterpart in the reference: an allocation-free form of his_grid_step. */
int32_t his_grid_step_noalloc(int32_t precision, const his_solver_cfg* cfg, const his_grid_desc* grid,
                              const his_step_params* params, double* vols, void* stream);

/* One member's 1-D channel network (flattened cells and faces; kinds 0 reach,
 * 1 junction, 2 inflow ghost, 3 stage ghost, 4 closed ghost).  Arrays are HOST
 * arrays copied at creation; A and Q are DEVICE float64 state (n_cells each).
 * Replaces hydrointel/solver/swe1d.py:113-166, :176-231 (Topology, SWE1D.__init__). */
typedef struct his_net_desc {
    int32_t n_cells, n_faces;
    const int32_t *kind, *ghost_src, *face_l, *face_r;
    const double* ghost_sign;
    const double *z, *manning, *dx;
    const double *b, *m, *yb, *ts;        /* cell sections */
    const double *fb, *fm, *fyb, *fts;    /* face sections */
    double *A, *Q;
} his_net_desc;

int32_t his_net_create(const his_solver_cfg* cfg, int32_t n_members, const his_net_desc* nets, his_net** out);
int32_t his_net_destroy(his_net* net);

/* n_sub 1-D substeps of dt/n_sub each for every member.  forcing: host array
 * n_members x n_sub x 2 (inflow m^3/s, stage m) at the substep start times.  If vols
 * is non-NULL it receives n_members x 3 float64 (bnd_in, bnd_out, clip) summed over
 * the substeps and the call synchronises.
 * Replaces hydrointel/solver/swe1d.py:265-368 (SWE1D._fill_ghosts / step / _step_core)
 * and the substep loop of hydrointel/solver/coupling.py:216-221. */
int32_t his_net_step(his_net* net, double dt, int32_t n_sub, const double* forcing, double* vols, void* stream);

/* Per-member 1-D CFL rate max over wet interior cells of (|u| + sqrt(gA/T))/dx and
 * whether any cell is wet (host outs; synchronises).
 * Replaces hydrointel/solver/swe1d.py:253-262 (SWE1D.max_dt). */
int32_t his_net_max_rate(his_net* net, double* rate, int32_t* any_wet, void* stream);

/* his_net_step_async: as his_net_step (forcing from any host memory, staged); vols
 * (n_members x 3) may be NULL.  Replaces the substep loop of
 * hydrointel/solver/coupling.py:216-221, which adds device tensors. */
int32_t his_net_step_async(his_net* net, double dt, int32_t n_sub, const double* forcing, double* vols,
                           void* stream);

/* n_sub 1-D substeps (his_net_step_async's arguments and asynchrony) adding their
 * boundary volumes and clip into rows 4, 5 and 7 of the DEVICE ledger described at
 * his_grid_step_ledger_async.  Replaces the per-substep MassBalance.add of bnd1d_in,
 * bnd1d_out and clip (hydrointel/solver/coupling.py:219-224). */
int32_t his_net_step_ledger_async(his_net* net, double dt, int32_t n_sub, const double* forcing, double* ledger,
                                  void* stream);

/* his_net_max_rate_async: per member (rate, wet) into rate_wet (n_members x 2; wet is
 * 1.0 when any interior cell is wet, else 0.0).  Replaces the reductions of
 * hydrointel/solver/swe1d.py:253-262. */
int32_t his_net_max_rate_async(his_net* net, double* rate_wet, void* stream);

/* Per-member channel volume sum(A*dx) over interior cells (host out; synchronises).
 * Replaces hydrointel/solver/swe1d.py:245-247 (SWE1D.volume). */
int32_t his_net_volume(his_net* net, double* vol, void* stream);

/* Weir links between a grid set and a network set (member i of each).  HOST arrays,
 * per member, copied at creation: cell1d, inv (-> unique cell), uniq (flat 2-D index
 * of each unique linked cell), zbank, length, z2.
 * Replaces hydrointel/solver/coupling.py:47-70 (Links, build_links). */
typedef struct his_links_desc {
    int32_t n_links, n_unique;
    const int32_t *cell1d, *inv;
    const int64_t* uniq;
    const double *zbank, *length, *z2;
} his_links_desc;

int32_t his_links_create(his_grid* grid, his_net* net, int32_t n_members, const his_links_desc* links,
                         his_links** out);
int32_t his_links_destroy(his_links* links);

/* Villemonte weir exchange for every member, applied in place to the 2-D depth and
 * momenta and the 1-D area.  cfg supplies weir_cw, exchange_limit and
 * exchange_relax for this call (NULL = the grid set's constants).  If V is non-NULL
 * it receives the per-link volumes (members concatenated, + = 2-D -> 1-D) and the
 * call synchronises.  Replaces hydrointel/solver/coupling.py:73-124 (exchange). */
int32_t his_exchange(his_links* links, const his_solver_cfg* cfg, double dt, double* V, void* stream);

/* his_exchange_async: as his_exchange; V (total links, device or page-locked host
 * memory) may be NULL.  The reference's exchange returns V as a device tensor
 * (hydrointel/solver/coupling.py:73-124). */
int32_t his_exchange_async(his_links* links, const his_solver_cfg* cfg, double dt, double* V, void* stream);

/* Running per-member totals of exchanged volume since creation or the last reset:
 * n_members x 2 (2-D -> 1-D, 1-D -> 2-D), host out, synchronises.  reset != 0 zeroes
 * them afterwards.  Replaces the exchange tallies of hydrointel/solver/coupling.py:210-211. */
int32_t his_links_exchanged(his_links* links, double* totals, int32_t reset, void* stream);

/* ------------------------------------------------------------------ engine */
/* Per-member forcing of the device-resident engine (host arrays copied at creation):
 * piecewise-constant rain blocks (m/s) from rain_t0 in blocks of rain_step seconds;
 * a harmonic tide base + sum amp cos(w (t + shift) - phase) (used by stage edges and
 * the 1-D stage end); a linearly interpolated inflow hydrograph (m^3/s, used by the
 * 1-D inflow end); and per 2-D edge a value source: 0 constant edge_val, 1 the
 * tide, 2 inflow x edge_val (a discharge per unit width).
 * Replaces hydrointel/engine.py:104-166 (BatchForcing), hyetograph.py:42-46,
 * tide.py:29-31, catchment.py:32-40. */
typedef struct his_forcing_desc {
    double t0, t_end;
    double rain_t0, rain_step;
    int32_t rain_n, tide_on;
    const double* rain;
    int32_t tide_n, q_n;
    double tide_base, tide_shift;
    double tide_amp[4], tide_w[4], tide_phase[4];
    double q_t0, q_step;
    const double* q;
    int32_t edge_src[4];
    double edge_val[4];
    /* Output (n_out = 0: none).  Output times are k * out_dt, k = 0 .. n_out - 1, each
     * at most t_end; every step is cut short at the next output time, and the state
     * reached there is written to slot k of DEVICE float32 arrays: snap_h, snap_u,
     * snap_v (n_out x ny x nx: depth and KP velocities) and, with a network, snap_eta,
     * snap_q (n_out x n_cells: level z + depth and discharge); snap_t (DEVICE float64,
     * n_out) receives the times and snap_ledger (DEVICE float64, n_out x 10, may be NULL)
     * the volume ledger: 2-D surface, 1-D channel and retained volume, then the
     * accumulated rain, infiltration, bnd2d_in, bnd2d_out, bnd1d_in, bnd1d_out and clip
     * (m^3).  Slot 0 (the initial state) is the caller's.
     * Replaces the output loop of hydrointel/solver/coupling.py:229-286 (snapshot,
     * run with out_times) and the output times of hydrointel/engine.py:48-50. */
    double out_dt;
    int32_t n_out, pad;
    float *snap_h, *snap_u, *snap_v, *snap_eta, *snap_q;
    double *snap_t, *snap_ledger;
} his_forcing_desc;

/* What the host reads back per member. status: 0 running, 1 done, 2 non-finite
 * state, 3 implausible state (2-D depth > 10 m), 4 more 1-D substeps than allowed.
 * acc: float64 volume totals (rain, infiltration, bnd2d_in, bnd2d_out, bnd1d_in,
 * bnd1d_out, clip) in m^3, in the reference's mass-balance terms. */
typedef struct his_member_report {
    double t, dt_last, dt_min, dt_max, rate;
    int64_t steps;
    int32_t status, n_sub_max, n_dt_clamped, outputs;   /* outputs: output slots written (incl. slot 0) */
    double acc[7];
} his_member_report;

typedef struct his_engine his_engine;

/* Device-resident coupled time loop over a grid set and (optionally) a network set
 * with links: every member advances with its own CFL dt until its t_end, forcing,
 * exchange, 1-D substeps, 2-D step and accounting all on the device, captured as
 * CUDA graphs of graph_steps steps (0 = default).  max_sub bounds the 1-D substeps
 * per step (0 = 64).  Replaces the per-step host loop of
 * hydrointel/solver/coupling.py:201-286 (CoupledEngine.step / run). */
int32_t his_engine_create(his_grid* grid, his_net* net, his_links* links, int32_t n_members,
                          const his_forcing_desc* forcing, int32_t max_sub, int32_t graph_steps, his_engine** out);
int32_t his_engine_destroy(his_engine* engine);

/* Enqueue n_steps steps of every running member on `stream` (asynchronous).  The
 * members run as independent chains (his_engine_set_chains), each on its own streams
 * and graphs; they join `stream` at the end of the call. */
int32_t his_engine_advance(his_engine* engine, int32_t n_steps, void* stream);

/* Capture, without running them, the CUDA graphs an advance of n_steps steps
 * launches: one graph of graph_steps steps per chain and one of the remaining
 * n_steps % graph_steps steps (one remainder size is kept at a time; an advance with
 * another remainder captures anew).  his_engine_advance captures what is missing
 * itself; calling this first keeps the capture out of a timed or latency-critical
 * advance.  No reference counterpart (the reference has no graphs). */
int32_t his_engine_prepare(his_engine* engine, int32_t n_steps);

/* Split the members into n_chains (1..8, at most one per member) independent chains
 * of about equal 2-D work, each advanced on its own streams and CUDA graphs, so that
 * one chain's latency-bound per-step kernels (dt, exchange, forcing, accounting)
 * overlap another's 2-D stages.  Results do not depend on the split (every member's
 * arithmetic is the same).  Default at creation: his_engine_default_chains (64 members
 * of 400 x 325 cells in 58 x 48 tiles: 8).  Waits for the engine's streams; graphs are
 * recaptured by the next advance.
 * No reference counterpart (the reference steps one batch with one shared dt). */
int32_t his_engine_set_chains(his_engine* engine, int32_t n_chains);
int32_t his_engine_chains(const his_engine* engine);
/* The default chain count for n_members members in n_tiles strip-chunk tiles: one per
 * 256 tiles, at least 1, at most 8 and at most n_members. */
int32_t his_engine_default_chains(int32_t n_members, int32_t n_tiles);

/* Per-member reports (host out, n_members; synchronises). */
int32_t his_engine_report(his_engine* engine, his_member_report* reports, void* stream);

/* Continue members from earlier reports: clock, last/min/max dt, CFL rate, step
 * count, status, substep and clamp statistics and the seven accumulators are set from
 * reports[m] for every member with mask[m] != 0 (mask NULL = all), so a member moved
 * into a new engine (another batch) carries on exactly where it stopped; its state
 * arrays are the ones its descriptors point to.  Synchronises.
 * Replaces the restart of hydrointel/solver/coupling.py:244-286 (CoupledEngine.run
 * with t0 and an existing MassBalance). */
int32_t his_engine_resume(his_engine* engine, const his_member_report* reports, const int32_t* mask, void* stream);

/* Run n_steps steps without graphs, bracketing each kernel class with CUDA events on
 * the stream it is launched on, and return the summed device milliseconds per class:
 * ms[0] pre (dt, exchange, forcing), ms[1] 2-D stage 1, ms[2] 2-D stage 2 + sources,
 * ms[3] 1-D substeps, ms[4] post (accounting), ms[5] whole steps.  Synchronises.
 * No reference counterpart: the measurement hook of the roofline report. */
int32_t his_engine_profile(his_engine* engine, int32_t n_steps, double* ms, void* stream);

#ifdef __cplusplus
}
#endif
#endif /* HIS_GB300_H */
