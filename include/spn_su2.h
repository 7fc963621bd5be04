/*
 * spn_su2.h — C ABI of the GB300 SU(2) pf-FRG flow core (libspn_su2.so).
 *
 * The library replaces, for one SpinParser flow, the work that the reference runs inside
 * SU2FrgCore (src/SU2/SU2FrgCore.cpp) through its LoadManager, and the correlation
 * measurement of SU2MeasurementCorrelation (src/SU2/SU2MeasurementCorrelation.cpp).
 * Host code above this ABI (the C++ FrgCore mirror in the package, or any FFI caller)
 * owns the cutoff loop, checkpoints and output files, as SpinParser::runCore does.
 *
 * Conventions
 *   - Every function returns 0 on success or a negative status (SPN_E_*); the message of
 *     the last failure on the calling thread is available through spn_last_error().
 *   - No C++ exception crosses this boundary.
 *   - Pointers named host_* / plain arrays are host memory; the library copies them.
 *   - Vertex arrays use the reference layout: index ((s*(s+1)/2 + u) * N + t) * Nl + rid,
 *     s >= u, i.e. SU2VertexTwoParticle::_dataSS/_dataDD (src/SU2/SU2VertexTwoParticle.hpp:603).
 */
#ifndef SPN_SU2_H
#define SPN_SU2_H

#include <stddef.h>

#ifdef __cplusplus
extern "C" {
#endif

/* status codes */
#define SPN_OK 0
#define SPN_E_ARGUMENT (-2)
#define SPN_E_INIT (-3)
#define SPN_E_IO (-4)
#define SPN_E_CUDA (-5)
#define SPN_E_DEVICE (-6)
#define SPN_E_INTERNAL (-7)
#define SPN_E_UNSUPPORTED (-8)

/* Copies the message of the last failed call on this thread into buf (NUL-terminated,
 * truncated to len).  Returns the full message length. */
int spn_last_error(char *buf, size_t len);

/* Library / device information: number of CUDA devices visible (0 without a GPU). */
int spn_device_count(int *count);
/* Free and total device memory in bytes (the admission budget of a serving loop). */
int spn_device_memory(int device, long long *free_bytes, long long *total_bytes);

/* Measured FP32 FMA throughput of a device (TFLOP/s, best of several runs of a pure-FFMA
 * kernel) and the SM clock it implies.  The vertex-flow kernel runs on the FP32 CUDA cores;
 * this is its roofline denominator.  No reference counterpart (benchmark support). */
int spn_measure_fp32_peak(int device, double *tflops, double *sm_clock_ghz_est);

/* Measured slab-gather rate of a device: segments of n_sites (<= 32) float2 pairs per second
 * that a pure gather kernel reads, one warp request per segment, at random starts among n_slabs
 * slabs (best of several runs; n_slabs sets the working set: F_N for a flow's vertex, a few
 * hundred for an L1-resident one).  The vertex flow's interpolation supports are such
 * segments; this is the denominator of its gather roofline.  No reference counterpart. */
int spn_measure_gather_peak(int device, int n_sites, int n_slabs, double *segments_per_s);

/* The frequency-mesh lookups of the vertex kernels, run on the host by the same code (diagnostics;
 * no device use).  pos: the n ascending positive mesh values.  lesser / greater: the mesh value of
 * FrequencyDiscretization::lesser / greater on the symmetric mesh (src/FrequencyDiscretization.hpp);
 * offset: FrequencyDiscretization::offset of |w|; lo, hi, bias: interpolateOffset of |w|.  Any
 * output may be NULL. */
int spn_mesh_probe(const float *pos, int n, float w, float *lesser, float *greater, int *offset, int *lo, int *hi,
                   float *bias);

/* The bucket index of the FP32 kernels' mesh lookups against binary search, on the host with the
 * kernels' code (diagnostics; no device use): *mismatches counts the w[k] for which the first
 * mesh index above (or at or above) w differs between the two. */
int spn_mesh_index_check(const float *pos, int n, const float *w, int count, int *mismatches);

/* One vertex read of the kernels on the host with their code (diagnostics; no device use), on a
 * state in the reference's layout (ss, dd: F_N * n_sites floats, element ((s(s+1)/2 + u) N + t)
 * n_sites + rid) and the pair's rid and exchanged rid: channel -1 getValue(..., None) (a direct
 * trilinear read), 0 / 1 / 2 an access buffer whose s / t / u coordinate is a mesh value
 * (generateAccessBuffer(s, t, u, S / T / U)), 3 the trilinear access buffer; density selects the
 * density or the spin vertex (src/SU2/SU2VertexTwoParticle.hpp:185-490). */
int spn_vertex_probe(const float *pos, int n, int n_sites, const float *ss, const float *dd, int rid12, int rid21,
                     float s, float t, float u, int channel, int density, float *value);

/* The self-energy read of the kernels (SU2VertexSingleParticle::getValue, odd in w and linearly
 * interpolated on the positive mesh) on the host with their code (diagnostics; no device use). */
int spn_self_energy_probe(const float *pos, int n, const float *data, float w, double *value);

/* The loop-frequency quadrature nodes of the node tables on the symmetric mesh, run on the host by
 * the same code (diagnostics; no device use): rule 0 ImplicitIntegrator's
 * integrateWithObscureLeftBoundary(min, last), 1 integrateWithObscureRightBoundary(beginNegative,
 * max), 2 integrateWithObscureBoundaries(min, max) (src/lib/Integrator.hpp:137-287).  The integral
 * of f is sum weight[i] * f(wp[i]).  Up to cap pairs are written; *count is the number of nodes. */
int spn_quadrature_nodes(const float *pos, int n, int rule, float min, float max, float *wp, double *weight, int cap,
                         int *count);

/* ------------------------------------------------------------------------------------
 * Host side: lattice / spin model (LatticeModelFactory::newLatticeModel,
 * src/LatticeModelFactory.cpp:733-1047) and discretisations (src/TaskFileParser.cpp:107-198).
 * These run on the CPU only and need no GPU.
 * ------------------------------------------------------------------------------------ */
typedef struct spn_lattice spn_lattice;

typedef struct {
    int n_sites;         /* Nl: number of representative site pairs (Lattice::size) */
    int n_sites_total;   /* all sites the lattice stores (Lattice::_dataSize) */
    int n_basis;         /* basis sites per unit cell */
    int n_range;         /* sites within range of basis site 0 (getRange(0)) */
    int n_overlap;       /* total RPA pairs, sum over rid of getOverlap(rid).size */
    int n_interactions;  /* couplings of the origin to representatives (SpinModel::interactions) */
} spn_lattice_info;

/* Builds the lattice named `lattice_name` from the unit cells in `resource_dir`, with
 * the spin model `model_name` whose coupling parameters are given as name/value strings
 * (values use the reference's number syntax, e.g. "1/sqrt(2)").
 * Replaces: LatticeUnitCell ctor (src/LatticeModelFactory.cpp:102), SpinModelUnitCell ctor
 * (:239) and newLatticeModel (:733). */
int spn_lattice_create(const char *resource_dir, const char *lattice_name, int range, const char *model_name,
                       int n_params, const char *const *param_names, const char *const *param_values,
                       spn_lattice **out);
int spn_lattice_destroy(spn_lattice *lat);
int spn_lattice_get_info(const spn_lattice *lat, spn_lattice_info *info);

/* Gather tables (any pointer may be NULL to skip that table):
 *   sites_rid[Nl]        Lattice::getSites()[j].rid            (src/Lattice.hpp:492)
 *   inv_sites_rid[Nl]    Lattice::getInvertedSites()[j].rid    (src/Lattice.hpp:481)
 *   overlap_ptr[Nl+1], overlap_rid1[n_overlap], overlap_rid2[n_overlap]
 *                        Lattice::getOverlap(rid).rid1/rid2    (src/Lattice.hpp:472)
 *   range_rid[n_range]   symmetryTransform(origin, j), j in getRange(0)
 *   range_inv_rid[n_range] symmetryTransform(j, origin)
 *   corr_rid[n_basis*n_range] symmetryTransform(basis b, j), j in getRange(b)
 *                        (the scatter of SU2MeasurementCorrelation.cpp:161-176)
 *   site_pos[3*n_basis*n_range] positions of getRange(b) sites (obs "meta/sites")
 *   basis_pos[3*n_basis], lattice_vectors[9]                   (obs "meta") */
int spn_lattice_get_tables(const spn_lattice *lat, int *sites_rid, int *inv_sites_rid, int *overlap_ptr,
                           int *overlap_rid1, int *overlap_rid2, int *range_rid, int *range_inv_rid, int *corr_rid,
                           double *site_pos, double *basis_pos, double *lattice_vectors);

/* Spin permutations of the same tables, for cores without SU(2) symmetry (XYZ): each entry is
 * an index p into the permutations (X,Y,Z) (X,Z,Y) (Y,X,Z) (Y,Z,X) (Z,X,Y) (Z,Y,X); component c
 * (0 = X, 1 = Y, 2 = Z) of a pair is component perm[p][c] of its representative
 * (LatticeSiteDescriptor::spinPermutation, src/Lattice.hpp:36-44, built in
 * LatticeModelFactory.cpp:833-870).  Arrays as in spn_lattice_get_tables: sites_perm and
 * inv_sites_perm [Nl], overlap_perm1 / overlap_perm2 [overlap_ptr[Nl]] (the pairs (0,j) and
 * (j,rid)), range_perm / range_inv_perm [n_range], corr_perm [n_basis * n_range].  For a model
 * whose couplings need no spin permutation every entry is 0. */
int spn_lattice_get_spin_tables(const spn_lattice *lat, int *sites_perm, int *inv_sites_perm, int *overlap_perm1,
                                int *overlap_perm2, int *range_perm, int *range_inv_perm, int *corr_perm);

/* All stored sites (Lattice::getSiteParameters, src/Lattice.hpp:397): site_params[4*i..] =
 * (a0, a1, a2, basis) of site id i, i < n_sites_total; and, if pair_rid is not NULL, the
 * full symmetry table pair_rid[i1*n_sites_total + i2] = symmetryTransform(i1, i2)
 * (-1 where the pair is out of range).  Diagnostics for the lattice KATs. */
int spn_lattice_get_sites(const spn_lattice *lat, int *site_params, int *pair_rid);

/* Interactions of the origin with representative rid: rid[n] and the 3x3 coupling matrix
 * (row-major, 9 floats each).  SpinModel::interactions (src/SpinModel.hpp). */
int spn_lattice_get_interactions(const spn_lattice *lat, int *rid, float *coupling);

/* The RPA schedule the device uses for a lattice (diagnostics; host only): the merged pair
 * lists of all rids cut into `lanes` balanced chunks (csrc/host/rpa_schedule.hpp; 1 <= lanes <=
 * 256: the device walks it with a warp's 32 lanes up to 32 sites, with the 128 or 256 threads of
 * a CTA above), the entries of each segment ordered against shared-memory bank collisions.
 * info[5] = {entries per lane, segments, total ints of sched, packed encoding (Nl <= 32),
 * row width of the outer-product matrix the packed entries index (0 otherwise)}.
 * With sched = NULL only info is filled; otherwise sched must hold info[2] ints, count and
 * slot_base `lanes` ints and seg_ptr Nl + 1 ints. */
int spn_rpa_schedule(int n_sites, const int *overlap_ptr, const int *overlap_rid1, const int *overlap_rid2, int lanes,
                     int *info, int *sched, int *count, int *slot_base, int *seg_ptr);

/* The per-site order of the RPA pairs of the XYZ (layout 0) or TRI (layout 1) core (diagnostics;
 * host only): order[overlap_ptr[j] .. overlap_ptr[j+1]) is a permutation of site j's pair
 * indices, chosen against shared-memory bank collisions of a walk with lane = site.  The vertex
 * kernels cut the site-ordered lists into 32 lane-balanced chunks and reorder the entries of each
 * run against the collisions of that walk (csrc/host/rpa_schedule.hpp, lane_schedule).
 * collisions[0] / [1]: collisions of the given order and of the chosen one (may be NULL). */
int spn_rpa_pair_order(int layout, int n_sites, const int *overlap_ptr, const int *overlap_rid1,
                       const int *overlap_rid2, const int *overlap_perm1, const int *overlap_perm2, int *order,
                       long long *collisions);

/* The lane-balanced walk of the XYZ (layout 1) or TRI (layout 2) vertex kernel's RPA pairs, or
 * the same chunking without the bank ordering (layout 0, last-entry bit 26) (diagnostics; host
 * only; csrc/host/rpa_schedule.hpp, lane_schedule): `words` are the site-ordered pair words
 * (site j's at overlap_ptr[j] .. overlap_ptr[j+1]), 32 lanes.  info[4] = {entries per lane,
 * segments, total ints of sched, last-entry bit}.  With sched = NULL only info is filled;
 * otherwise sched holds info[2] ints, count and slot_base 32 ints, seg_ptr Nl + 1 ints. */
int spn_rpa_lane_schedule(int layout, int n_sites, const int *overlap_ptr, const int *words, int *info, int *sched,
                          int *count, int *slot_base, int *seg_ptr);

/* Writes the lattice debug file (.ldf) as `--debugLattice`-free SpinParser always does. */
int spn_lattice_write_ldf(const spn_lattice *lat, const char *path);

/* Exponential frequency mesh: min * powf(powf(max/min, 1/(count-1)), i), i < count
 * (src/TaskFileParser.cpp:121-123).  out has room for `count` floats. */
int spn_frequency_exponential(float min, float max, int count, float *out);

/* A number of the task, lattice and model files (InputParser::stringToDouble,
 * src/lib/InputParser.hpp:24-56): sqrt(x) terms are evaluated first, then x*y and x/y left to
 * right, each result written back with 20 decimals, then the text is read as a double.  The
 * files' float values are (float) of it. */
int spn_parse_number(const char *text, double *value);

/* Exponential cutoff list: repeated float multiplication max, max*step, ... while > min
 * (src/TaskFileParser.cpp:171-176).  Writes at most `cap` values, *n receives the count
 * (which may exceed cap; call again with a larger buffer). */
int spn_cutoff_exponential(float max, float min, float step, float *out, int cap, int *n);

/* Initial condition of SU2EffectiveAction (src/SU2/SU2EffectiveAction.hpp:38-60): zeros,
 * then v4ss[it*Nl + rid] += J_xx(rid) / normalization for every frequency triple it. */
int spn_su2_initial_state(const spn_lattice *lat, int n_freq, float normalization, float *v2, float *v4ss,
                          float *v4dd);

/* ------------------------------------------------------------------------------------
 * Device side: one SU(2) flow resident in GPU memory.
 * ------------------------------------------------------------------------------------ */
typedef struct spn_su2 spn_su2;

/* Description of one flow; the library copies every table at create time. */
typedef struct {
    int n_freq;                 /* N positive Matsubara frequencies */
    const float *freq;          /* [N] ascending, positive (FrequencyDiscretization values) */
    int n_sites;                /* Nl */
    const int *sites_rid;       /* [Nl] */
    const int *inv_sites_rid;   /* [Nl] */
    const int *overlap_ptr;     /* [Nl+1] */
    const int *overlap_rid1;    /* [overlap_ptr[Nl]] */
    const int *overlap_rid2;    /* [overlap_ptr[Nl]] */
    int n_range;                /* sites in range of the origin */
    const int *range_rid;       /* [n_range] */
    const int *range_inv_rid;   /* [n_range] */
    int n_corr;                 /* n_basis * n_range entries of the correlation output */
    const int *corr_rid;        /* [n_corr] rid each correlation entry reads */
    float spin_length;          /* S (SU2FrgCore option "spin", default 0.5) */
    int device;                 /* CUDA device ordinal */
    int flags;                  /* SPN_SU2_* flags below */
} spn_su2_desc;

/* Self-energy and its flow are kept in FP64 on the device (plain mode keeps FP32, the
 * reference's type). */
#define SPN_SU2_FP64_SELF_ENERGY 0x1
/* The whole flow in FP64 on the device: state, flow, loop-frequency nodes, every integrand
 * and the measurement (the precision reference for FP32 flows of the same task; the cutoff
 * list and the frequency mesh keep the task's float values).  The float entry points convert
 * on the host; the _f64 entry points below move the double arrays themselves.  Such a flow is
 * evaluated by a plain FP64 kernel (one warp per frequency triple): correct, not fast.  Not
 * accepted by spn_batch_add. */
#define SPN_SU2_FP64 0x2

/* Creates a flow (allocates its device memory).  State starts at zero, cutoff 0.
 * Replaces SU2FrgCore's constructor (src/SU2/SU2FrgCore.cpp:17-81). */
int spn_su2_create(const spn_su2_desc *desc, spn_su2 **out);
int spn_su2_destroy(spn_su2 *h);

/* Work is queued on this stream (a cudaStream_t; NULL selects the library's own). */
int spn_su2_set_stream(spn_su2 *h, void *stream);

/* Sizes: N, Nl and F_N = N*N*(N+1)/2 (so each vertex array holds F_N*Nl floats). */
int spn_su2_get_sizes(const spn_su2 *h, int *n_freq, int *n_sites, long long *n_triples);

/* Copy the flowing state (EffectiveAction) in / out: cutoff, v2[N], v4ss/v4dd[F_N*Nl].
 * Replaces readCheckpoint / writeCheckpoint data movement (src/SU2/SU2EffectiveAction.hpp:79-205). */
int spn_su2_set_state(spn_su2 *h, float cutoff, const float *v2, const float *v4ss, const float *v4dd);
int spn_su2_get_state(spn_su2 *h, float *cutoff, float *v2, float *v4ss, float *v4dd);

/* Sets the cutoff of the flowing state without touching the vertex data (what
 * SpinParser does when it resumes from a checkpoint: EffectiveAction::cutoff, src/EffectiveAction.hpp:58). */
int spn_su2_set_cutoff(spn_su2 *h, float cutoff);

/* Number of loop-frequency nodes per transfer frequency used by the last compute_step
 * (counts[N]): conventional terms plus the trapezoid nodes of the Katanin integrals. */
int spn_su2_get_node_counts(spn_su2 *h, int *counts);

/* FrgCore::computeStep (src/SU2/SU2FrgCore.cpp:89-109): self-energy flow, then the
 * two-particle vertex flow, into the device-resident flow buffers.  Asynchronous. */
int spn_su2_compute_step(spn_su2 *h);

/* Picks the vertex-flow kernel variant for this flow by timing the candidates on the current
 * state (`reps` launches each): nodes a site group evaluates per iteration (1 or 2) and
 * whether the RPA schedule is staged in shared memory.  All variants give identical results.
 * Leaves the state unchanged; reports the choice and the persistent grid size.  Replaces the
 * reference LoadManager's throughput model (src/lib/LoadManager.hpp:796-852) as the tuning
 * step of the work distribution. */
int spn_su2_autotune(spn_su2 *h, int reps, int *npi, int *sched_in_smem, int *grid);

/* Selects a vertex-flow variant explicitly (npi = 1 or 2; schedule in shared memory or not).
 * SPN_E_UNSUPPORTED if it does not fit for this lattice. */
int spn_su2_set_variant(spn_su2 *h, int npi, int sched_in_smem);

/* Copies the flow computed by the last compute_step: dv2[N], dv4ss/dv4dd[F_N*Nl]. */
int spn_su2_get_flow(spn_su2 *h, float *dv2, float *dv4ss, float *dv4dd);

/* FrgCore::finalizeStep (src/SU2/SU2FrgCore.cpp:111-137): explicit Euler step of the
 * state by (new_cutoff - cutoff) * flow, then cutoff = new_cutoff.  Asynchronous. */
int spn_su2_finalize_step(spn_su2 *h, float new_cutoff);

/* SU2MeasurementCorrelation::_calculateCorrelation at the current cutoff (nu = 0):
 * zz[n_corr] and dd[n_corr] in the reference's (basis, site-in-range) order.  Either
 * pointer may be NULL.  chi_zz/chi_dd (may be NULL) receive the per-rid susceptibility. */
int spn_su2_measure_correlation(spn_su2 *h, float *zz, float *dd, float *chi_zz, float *chi_dd);

/* The same measurement split in two: launch (asynchronous, result stays on the device) and
 * copy-out of the last launched measurement (synchronises). */
int spn_su2_launch_correlation(spn_su2 *h);
int spn_su2_get_correlation(spn_su2 *h, float *zz, float *dd, float *chi_zz, float *chi_dd);

/* Double-precision state, flow and measurement of a flow created with SPN_SU2_FP64
 * (SPN_E_UNSUPPORTED for other flows); same layouts and meaning as the float calls above. */
int spn_su2_set_state_f64(spn_su2 *h, float cutoff, const double *v2, const double *v4ss, const double *v4dd);
int spn_su2_get_state_f64(spn_su2 *h, float *cutoff, double *v2, double *v4ss, double *v4dd);
int spn_su2_get_flow_f64(spn_su2 *h, double *dv2, double *dv4ss, double *dv4dd);
int spn_su2_measure_correlation_f64(spn_su2 *h, double *zz, double *dd, double *chi_zz, double *chi_dd);

/* Correlation measurement that allocates no device memory.  No counterpart in the reference:
 * it exists for callers that cannot allocate device memory when they measure, such as a host
 * framework that reserves the GPU's memory up front in its own pool (a cudaMalloc here would
 * fail or bypass its accounting) or a time-critical loop that must not enter the CUDA allocator.
 * Every pointer is DEVICE memory owned by the caller: freq[n_freq], sites_rid and
 * inv_sites_rid[n_sites], corr_rid[n_corr], the state v2[n_freq], v4ss and v4dd[F_N*n_sites],
 * and out[2*n_corr + 2*n_sites] which receives zz, dd, chi_zz and chi_dd as in
 * spn_su2_measure_correlation.  The kernels' scratch is a fixed array inside the library
 * (1 064 960 bytes per GPU, held until the process exits), which limits n_freq <= 256 and
 * n_sites <= 128; larger sizes are rejected with SPN_E_UNSUPPORTED.  The first call on a device
 * looks up that array's device address (with the device current) and should come before any
 * stream capture.  The looked-up address is kept for the life of the process: a
 * cudaDeviceReset() ends the context that holds the array, so after a reset this entry point
 * must not be called on that device again in the same process.  Work is queued on `stream` (a
 * cudaStream_t, NULL = default stream) and the call returns without waiting.  All calls on one
 * device share the array: calls whose work overlaps on the GPU race and must be ordered by the
 * caller.  The tables are read on the device and not checked on the host: sites_rid and
 * inv_sites_rid entries must lie in [0, n_sites); a corr_rid entry outside [0, n_sites) gives
 * NaN in its zz and dd outputs. */
int spn_su2_correlation_noalloc(int n_freq, const float *freq, int n_sites, const int *sites_rid,
                                const int *inv_sites_rid, int n_corr, const int *corr_rid, float spin_length,
                                float cutoff, const float *v2, const float *v4ss, const float *v4dd, float *out,
                                void *stream);

/* EffectiveAction::isDiverged on the last computed flow (any NaN).  Synchronises. */
int spn_su2_is_diverged(spn_su2 *h, int *diverged);

/* Waits for all queued work of this flow. */
int spn_su2_synchronize(spn_su2 *h);

/* Kernel timing with CUDA events recorded on the flow's stream around each compute_step
 * kernel.  enable != 0 starts recording (and clears the totals). */
int spn_su2_set_profiling(spn_su2 *h, int enable);
/* Totals since profiling was enabled: milliseconds and launches of the vertex-flow kernel
 * and of the whole compute_step (self-energy + tables + vertex). */
int spn_su2_get_profile(spn_su2 *h, double *vertex_ms, int *vertex_launches, double *step_ms, int *steps);

/* ------------------------------------------------------------------------------------
 * Batches: many flows on one GPU advanced together.  No reference counterpart (the
 * reference runs one flow per process); each flow follows SpinParser::runCore's cycle
 * (compute, measure, divergence check, Euler step; final measurement at the last cutoff).
 * A step launches every kernel once for all flows -- the vertex flow as one persistent launch
 * over the ragged list of all flows' frequency triples -- and, by default, replays the step
 * as a CUDA graph while the set of flows and their phases are unchanged.  Flows may be added
 * and removed between steps (continuous batching); each flow's results are bit-identical to
 * the same flow run alone with spn_su2_* and the same vertex-flow variant.
 * ------------------------------------------------------------------------------------ */
typedef struct spn_batch spn_batch;

#define SPN_PHASE_FLOWING 0 /* computing its flow */
#define SPN_PHASE_FINAL 1   /* at the last cutoff, final measurement pending */
#define SPN_PHASE_DONE 2    /* finished (see flags) */
#define SPN_FLOW_DIVERGED 0x1
#define SPN_FLOW_NODE_OVERFLOW 0x2

int spn_batch_create(int device, spn_batch **out);
int spn_batch_destroy(spn_batch *b);
/* Vertex-flow variant of the batch (npi = 1 or 2) and whether steps are replayed as graphs.
 * Variants do not change results. */
int spn_batch_set_variant(spn_batch *b, int npi, int use_graph);
/* Cross-flow sharing in the vertex flow.  Flows of a batch that have the same frequency mesh,
 * lattice tables, spin length and cutoff list and stand at the same cutoff (a parameter scan's
 * flows of one lattice, range and frequency count, admitted together) have the same
 * loop-frequency nodes and interpolation supports; groups of at least min_group such flows
 * (0 = off, the default; spn_batch_autotune may switch it on) are evaluated by a kernel that
 * builds each node's supports once per subgroup and evaluates them for all its flows.  Subgroups hold at most the kernel's flows
 * per block divided by cap_divisor (1, 2 or 4; default 1).  No counterpart in the reference,
 * which runs one flow per process.  Results are bit-identical to the per-flow kernel's. */
int spn_batch_set_grouping(spn_batch *b, int min_group, int cap_divisor);
/* Holds a flow out of the following steps (paused = 1) or lets it take part again (0).  A
 * paused flow keeps its state, phase and results; a serving loop uses this to give the GPU to
 * the flows with the least remaining work.  Results do not change. */
int spn_batch_set_paused(spn_batch *b, int flow_id, int paused);
/* Flows the current plan evaluates with the grouped kernel. */
int spn_batch_grouped_flows(spn_batch *b, int *n_grouped);
/* Batch autotuner: times the vertex flow of the current flows, `reps` launches per candidate,
 * over nodes per iteration (1, 2) x RPA schedule staging (without sharing) and, if sharing is
 * enabled (spn_batch_set_grouping), x sharing (full or half subgroups), and keeps the fastest
 * (returned, with its time per launch in ms).
 * Touches no flow's state or results; call it between steps, after the flows of interest are
 * admitted.  Replaces the reference LoadManager's chunk-size choice
 * (src/lib/LoadManager.hpp:796-852). */
int spn_batch_autotune(spn_batch *b, int reps, int *npi, int *min_group, int *cap_divisor, float *best_ms);
/* Device memory a flow takes in a batch (state, flow, tables, measurement history): the
 * admission measure of a serving loop. */
int spn_batch_footprint(const spn_su2_desc *desc, int n_cutoffs, long long *bytes);
/* Admits a flow with its cutoff list (descending) and initial state at cutoffs[0]; returns its
 * id.  desc->device must be the batch's device. */
int spn_batch_add(spn_batch *b, const spn_su2_desc *desc, int n_cutoffs, const float *cutoffs, const float *v2,
                  const float *v4ss, const float *v4dd, int *flow_id);
/* Advances every unfinished flow by one step (asynchronous); *n_active receives the number of
 * flows not yet done as far as the host knows (divergence is learnt one step later). */
int spn_batch_step(spn_batch *b, int *n_active);
/* Waits for all queued steps and refreshes the host's view of every flow. */
int spn_batch_synchronize(spn_batch *b);
/* Phase, cutoff index and SPN_FLOW_* flags of a flow as the host last saw them. */
int spn_batch_poll(spn_batch *b, int flow_id, int *phase, int *step, int *flags);
/* Measurements recorded so far (waits for queued work): *n_measured rows of cutoffs[k],
 * zz/dd[k][n_corr] and chi_zz/chi_dd[k][Nl], the outputs of spn_su2_measure_correlation at
 * every cutoff the flow reached.  Any output pointer may be NULL. */
int spn_batch_get_result(spn_batch *b, int flow_id, int *n_measured, float *cutoffs, float *zz, float *dd,
                         float *chi_zz, float *chi_dd);
/* Current state of a flow (waits for queued work). */
int spn_batch_get_state(spn_batch *b, int flow_id, float *cutoff, float *v2, float *v4ss, float *v4dd);
/* Releases a flow's device memory; its id may be reused by a later spn_batch_add. */
int spn_batch_remove(spn_batch *b, int flow_id);
/* Steps run, CUDA graphs built, flows held. */
int spn_batch_stats(spn_batch *b, long long *steps, long long *graph_builds, int *n_flows);

/* ------------------------------------------------------------------------------------
 * Files: checkpoints and observables in the reference's HDF5 layout.  Host only.
 * ------------------------------------------------------------------------------------ */

/* SU2EffectiveAction::writeCheckpoint (src/SU2/SU2EffectiveAction.hpp:79-147): group
 * "checkpoint_<id>" with attribute "cutoff" and datasets cutoff[1], v2[n_v2], v4dd[n_v4],
 * v4ss[n_v4].  append != 0 adds to an existing file (a new file otherwise); *checkpoint_id
 * receives the new id, or -1 when the file already holds a checkpoint at this cutoff (nothing
 * is written then). */
int spn_su2_write_checkpoint(const char *path, int append, float cutoff, int n_v2, const float *v2, long long n_v4,
                             const float *v4ss, const float *v4dd, int *checkpoint_id);

/* SU2EffectiveAction::readCheckpoint (src/SU2/SU2EffectiveAction.hpp:149-200): reads group
 * "checkpoint_<checkpoint_id>", or with checkpoint_id < 0 the checkpoint named after the
 * index of the last group.  *found = 0 when that group or one of its datasets is missing.
 * SPN_E_IO if the file cannot be read; SPN_E_ARGUMENT if its sizes differ from n_v2 / n_v4. */
int spn_su2_read_checkpoint(const char *path, int checkpoint_id, float *cutoff, int n_v2, float *v2, long long n_v4,
                            float *v4ss, float *v4dd, int *found);

/* SU2MeasurementCorrelation::takeMeasurement's file output (src/SU2/SU2MeasurementCorrelation.cpp:179-355):
 * adds zz and dd ([n_basis][n_range] of the lattice) as measurement groups of "SU2CorZZ" and
 * "SU2CorDD" in the observable file, writing the "meta" group (lattice vectors, basis,
 * sites) where it is missing.  *written = 0 when a measurement at this cutoff exists (it is
 * kept and the new one discarded, as the reference does). */
int spn_su2_write_correlation(const char *path, const spn_lattice *lat, float cutoff, const float *zz, const float *dd,
                              int *written);

/* ------------------------------------------------------------------------------------
 * Task driver: SpinParser::run / runCore (src/SpinParser.cpp:53-210) for SU(2) tasks on
 * one GPU.  Parses the task file (src/TaskFileParser.cpp), builds the lattice, writes the
 * .ldf, runs the cutoff loop on the device with checkpoints, measurements, deferred
 * measurements and the post-processing stage, and writes the calculation status back into
 * the task file.  Output files sit beside the task file (.obs, .checkpoint, .data, .ldf).
 * ------------------------------------------------------------------------------------ */
typedef struct {
    const char *resource_path; /* directory with the lattice / model XML files; NULL = the package's res/ */
    int checkpoint_time;       /* seconds between checkpoints (--checkpointTime, default 3600) */
    int force_restart;         /* --forceRestart */
    int defer;                 /* --defer: archive the vertex for all measurements */
    int debug_lattice;         /* --debugLattice: stop after the lattice (no GPU needed) */
    int verbose;               /* -1 errors and warnings only, 0 progress, 1 debug (--verbose) */
    int device;                /* CUDA device ordinal */
    int flags;                 /* spn_su2_desc flags */
    int autotune;              /* pick the vertex-flow variant by timing before the loop */
} spn_run_options;

typedef struct {
    int status;            /* final calculation status: 0 new, 1 running, 2 postprocessing, 3 finished */
    int steps;             /* flow steps computed (compute_step + finalize_step) */
    int measurements;      /* correlation measurements evaluated on the device */
    int diverged;          /* the flow stopped on a NaN */
    double flow_seconds;   /* wall time of the cutoff loop */
} spn_run_result;

/* Fills o with the reference's defaults (checkpoint_time 3600, all switches off, device 0). */
int spn_run_options_default(spn_run_options *o);
/* Runs a task file; result may be NULL. */
int spn_run_task(const char *task_path, const spn_run_options *o, spn_run_result *result);

/* ------------------------------------------------------------------------------------
 * XYZ core: models with diagonal, possibly anisotropic couplings (Heisenberg-Kitaev, XXZ, ...)
 * on the same skeleton, with four vertex components X, Y, Z and density D
 * (src/XYZ/XYZFrgCore.cpp, XYZVertexTwoParticle.hpp, XYZMeasurementCorrelation.cpp).
 * Arrays in the reference layout: v2[N], v4xx/v4yy/v4zz/v4dd[F_N*Nl].
 * ------------------------------------------------------------------------------------ */
typedef struct spn_xyz spn_xyz;

typedef struct {
    int n_freq;                 /* N */
    const float *freq;          /* [N] ascending, positive */
    int n_sites;                /* Nl <= 128 */
    const int *sites_rid, *sites_perm;         /* [Nl] getSites(): rid and spin permutation */
    const int *inv_sites_rid, *inv_sites_perm; /* [Nl] getInvertedSites() */
    const int *overlap_ptr;     /* [Nl+1] */
    const int *overlap_rid1, *overlap_rid2;    /* [overlap_ptr[Nl]] */
    const int *overlap_perm1, *overlap_perm2;  /* [overlap_ptr[Nl]] permutations of (0,j), (j,rid) */
    int n_range;
    const int *range_rid, *range_inv_rid;      /* [n_range] */
    int n_corr;                 /* n_basis * n_range */
    const int *corr_rid, *corr_perm;           /* [n_corr] */
    int device;
    int flags;                  /* reserved, 0 */
} spn_xyz_desc;
/* Permutation indices are those of spn_lattice_get_spin_tables. */

/* XYZEffectiveAction initial condition (src/XYZ/XYZEffectiveAction.hpp:38-60): zeros, then
 * v4cc[it*Nl + rid] += 0.25 J^cc(rid) / normalization for c = x, y, z. */
int spn_xyz_initial_state(const spn_lattice *lat, int n_freq, float normalization, float *v2, float *v4xx,
                          float *v4yy, float *v4zz, float *v4dd);

/* The flow cycle, as the spn_su2_* calls (XYZFrgCore::computeStep / finalizeStep,
 * XYZFrgCore.cpp:109-159). */
int spn_xyz_create(const spn_xyz_desc *desc, spn_xyz **out);
int spn_xyz_destroy(spn_xyz *h);
int spn_xyz_set_state(spn_xyz *h, float cutoff, const float *v2, const float *v4xx, const float *v4yy,
                      const float *v4zz, const float *v4dd);
int spn_xyz_get_state(spn_xyz *h, float *cutoff, float *v2, float *v4xx, float *v4yy, float *v4zz, float *v4dd);
int spn_xyz_compute_step(spn_xyz *h);
int spn_xyz_get_flow(spn_xyz *h, float *dv2, float *v4xx, float *v4yy, float *v4zz, float *v4dd);
int spn_xyz_finalize_step(spn_xyz *h, float new_cutoff);
/* Correlations xx/yy/zz/dd[n_corr] in the (basis, site-in-range) order of XYZCorXX etc.
 * (XYZMeasurementCorrelation.cpp:166-184) and chi[4][Nl] per representative; any pointer may be
 * NULL. */
int spn_xyz_measure_correlation(spn_xyz *h, float *xx, float *yy, float *zz, float *dd, float *chi);
int spn_xyz_is_diverged(spn_xyz *h, int *diverged);

/* One vertex read of the XYZ kernels on the host with their code (diagnostics; no device use), on
 * a state in the layout of spn_xyz_set_state (v4xx ... v4dd: F_N * n_sites floats each), for the
 * pair with rid rid12 and spin permutation perm12 and the site-exchanged pair (rid21, perm21):
 * value[4] = X, Y, Z, D.  channel -1: getValue(..., None) (a direct trilinear read; identity
 * permutations); 0 / 1 / 2: the superbundle gather through an access buffer whose s / t / u
 * coordinate is a mesh value; 3: the correlation's gather through the trilinear access buffer.
 * local != 0 (channels 0-3): getValueLocal instead of the pair's read
 * (src/XYZ/XYZVertexTwoParticle.hpp:185-612). */
int spn_xyz_vertex_probe(const float *pos, int n, int n_sites, const float *v4xx, const float *v4yy,
                         const float *v4zz, const float *v4dd, int rid12, int rid21, int perm12, int perm21, float s,
                         float t, float u, int channel, int local, float *value);

/* ------------------------------------------------------------------------------------
 * TRI core: time-reversal-invariant models with general, also off-diagonal, couplings
 * (Heisenberg-Kitaev-Gamma, ...), 16 vertex components (a, b), a, b in X, Y, Z, density
 * (src/TRI/TRIFrgCore.cpp, TRIVertexTwoParticle.hpp, TRIMeasurementCorrelation.cpp).
 * Arrays in the reference layout: v2[N], v4[F_N][16][Nl] (component 4a + b), the checkpoint
 * dataset "v4" of TRIEffectiveAction (TRIEffectiveAction.hpp:147-148).
 * ------------------------------------------------------------------------------------ */
typedef struct spn_tri spn_tri;
typedef spn_xyz_desc spn_tri_desc; /* the same lattice and spin-permutation tables */

/* TRIEffectiveAction initial condition (src/TRI/TRIEffectiveAction.hpp:38-62): zeros, then
 * v4[it][a][b][rid] += 0.25 J^ab(rid) / normalization for spin components a, b. */
int spn_tri_initial_state(const spn_lattice *lat, int n_freq, float normalization, float *v2, float *v4);

/* The flow cycle (TRIFrgCore::computeStep / finalizeStep, TRIFrgCore.cpp:76-120). */
int spn_tri_create(const spn_tri_desc *desc, spn_tri **out);
int spn_tri_destroy(spn_tri *h);
int spn_tri_set_state(spn_tri *h, float cutoff, const float *v2, const float *v4);
int spn_tri_get_state(spn_tri *h, float *cutoff, float *v2, float *v4);
int spn_tri_compute_step(spn_tri *h);
int spn_tri_get_flow(spn_tri *h, float *dv2, float *dv4);
int spn_tri_finalize_step(spn_tri *h, float new_cutoff);
/* Correlations corr[10][n_corr] in the order XX XY XZ YX YY YZ ZX ZY ZZ DD, each in the
 * (basis, site-in-range) order of TRICorXX etc. (TRIMeasurementCorrelation.cpp:255-283), and
 * chi[16][Nl] per representative (the mixed spin/density components are zero); either
 * pointer may be NULL. */
int spn_tri_measure_correlation(spn_tri *h, float *corr, float *chi);
int spn_tri_is_diverged(spn_tri *h, int *diverged);

/* One vertex read of the TRI kernels on the host with their code (diagnostics; no device use), on
 * a state v4 in the reference layout, with the arguments of spn_xyz_vertex_probe: value[16] =
 * component 4a + b.  channel -1: getValue(..., a, b, None); 0 / 1 / 2: the vertex kernel's slab
 * gather through an access buffer whose s / t / u coordinate is a mesh value; 3: the
 * correlation's superbundle read through the trilinear access buffer; local != 0: getValueLocal
 * (src/TRI/TRIVertexTwoParticle.hpp:190-671). */
int spn_tri_vertex_probe(const float *pos, int n, int n_sites, const float *v4, int rid12, int rid21, int perm12,
                         int perm21, float s, float t, float u, int channel, int local, float *value);

/* The coefficient tables the TRI kernels evaluate, as rows (table, output, n, a, b, sign):
 * table 0 particle-particle ladder, 1 particle-hole ladder, 2 RPA, 3 chalice, 4 inverse
 * chalice, 5 egg diagram; 1152 rows of 6 ints.  Host only (no device needed). */
int spn_tri_tables(int *rows);

#ifdef __cplusplus
}
#endif

#endif /* SPN_SU2_H */
