/*
 * bh_gpu.h -- C ABI of the GB300 Barnes-Hut engine (libbh_gpu.so).
 *
 * Drop-in boundary for the single-rank `--fc tree` force path of
 * YonatanGM/Barnes-Hut.  Every entry point takes plain pointers and sizes,
 * returns an int status (BH_OK == 0) and never throws.  The last error
 * message of the calling thread is available from bh_last_error().
 *
 * Array conventions (identical to the reference's body.h:4-10 Vec3 AoS):
 *   pos, vel, acc : n*3 doubles, x,y,z per body
 *   mass          : n doubles
 *   ids, keys     : n uint64
 *   bbox          : {min.x, min.y, min.z, max.x, max.y, max.z}
 *                   (BoundingBox, include/bounding_box.h:11-22)
 * Units are the reference's: AU, day, kg; G = 1.48812e-34 (src/main.cpp:174).
 *
 * Each line below names the reference interface (file:line) an entry point
 * replaces.  Entry points with no reference counterpart say so.
 */
#ifndef BH_GPU_H
#define BH_GPU_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define BH_API_VERSION 1

/* ---- status codes ---------------------------------------------------- */
enum bh_status {
    BH_OK = 0,
    BH_ERR_INVALID_ARGUMENT = 1, /* null pointer, negative size, theta < 0 ... */
    BH_ERR_CUDA = 2,             /* a CUDA runtime call failed                 */
    BH_ERR_OUT_OF_MEMORY = 3,    /* device or host allocation failed           */
    BH_ERR_CAPACITY = 4,         /* more bodies than the context was made for  */
    BH_ERR_OVERFLOW = 5,         /* traversal stack/list overflow flag (the
                                    reference throws "BH stack overflow",
                                    src/traversal.cpp:94)                      */
    BH_ERR_TIMEOUT = 6,          /* a bounded device-side wait gave up         */
    BH_ERR_NONFINITE = 7,        /* a position is NaN or infinite              */
    BH_ERR_STATE = 8,            /* call out of order (e.g. forces before tree)*/
    BH_ERR_IO = 9,               /* file cannot be opened                      */
    BH_ERR_NO_DEVICE = 10        /* no CUDA device                             */
};

/* ---- force modes ----------------------------------------------------- */
enum bh_mode {
    /* The reference's criterion and arithmetic: FP64, IEEE sqrt/div, no
     * contraction, interactions summed in the reference's DFS order, so
     * accelerations equal computeAccelerations (src/traversal.cpp:13-103)
     * bit for bit. */
    BH_MODE_PLAIN_FP64 = 0,
    /* Same interaction set as BH_MODE_PLAIN_FP64: the warp's group box
     * classifies nodes, undecided ones get each body's exact FP64 test, and
     * lane masks carry which bodies still need a subtree.  Interactions are
     * evaluated in FP64 from shared-memory lists with rsqrt and FMA, so
     * results agree with the reference to ~1e-15 relative, not bit for bit.
     * No reference counterpart. */
    BH_MODE_FP64_LIST = 1,
    /* Far field in FP32 on displacements formed in FP64 relative to the
     * warp's group centre; FP32 partials summed into FP64 accumulators; the
     * Sun and planets (the BH_NUM_MASSIVE heaviest bodies) summed directly in
     * FP64 and excluded from the far-field tree.  No reference counterpart. */
    BH_MODE_FP32_FAR = 2,
    /* BH_MODE_FP32_FAR with the learned acceptance criterion (see
     * bh_learned_*).  No reference counterpart. */
    BH_MODE_LEARNED = 3,
    /* BH_MODE_FP32_FAR with one acceptance decision per warp group of 32
     * Morton-consecutive bodies: a node is accepted for the whole group when
     * every body's own theta test (src/traversal.cpp:78) accepts it, and
     * opened for the whole group otherwise.  Each body's interaction set is
     * then at least as fine as its own test at the same theta gives (more
     * accurate, more interactions per body), and every staged node is
     * evaluated for all the warp's lanes, none masked.  No reference
     * counterpart. */
    BH_MODE_FP32_GROUP = 4
};

#define BH_MAX_DEPTH 21   /* reference MAX_L / MAX_DEPTH (traversal.cpp:28) */
#define BH_NUM_MASSIVE 9  /* Sun + 8 planets: direct FP64 terms in FP32 modes */

const char *bh_last_error(void);
const char *bh_status_string(int status);
int bh_api_version(void);

/* ---- device-resident context ---------------------------------------- */
/* A context owns all device buffers for up to `capacity` bodies on one GPU
 * and one CUDA stream; the body state stays on the device across steps.
 * No reference counterpart (the reference keeps std::vectors in main.cpp). */
typedef struct bh_context bh_context;

int bh_context_create(int64_t capacity, int device, bh_context **out);
int bh_context_destroy(bh_context *ctx);
/* Blocks until all work queued on the context's stream has finished and
 * reports any error flag a kernel raised. */
int bh_context_sync(bh_context *ctx);
/* The context's cudaStream_t, for callers that order their own work. */
int bh_context_stream(bh_context *ctx, void **stream_out);

/* Upload host arrays (any of vel/mass/ids may be NULL only if n == 0).
 * Resets the accumulated time to 0 and the stored accelerations to 0, as
 * the reference's main.cpp:175,178 do before the loop. */
int bh_set_bodies(bh_context *ctx, int64_t n, const double *pos, const double *vel,
                  const double *mass, const uint64_t *ids);
/* Upload the accelerations of the previous step (n*3), for a caller that
 * keeps the whole state on the host between steps (the first half kick of
 * the next step uses them, src/main.cpp:193-200). */
int bh_set_accelerations(bh_context *ctx, const double *acc);
/* Download the state in its current (last sorted) order; NULL skips. */
int bh_get_bodies(bh_context *ctx, double *pos, double *vel, double *mass, uint64_t *ids, double *acc);
int bh_num_bodies(bh_context *ctx, int64_t *n_out);

/* ---- the hot path, stage by stage ------------------------------------ */
/* compute_local_bbox (src/bounding_box.cpp:23-44); on one rank
 * compute_global_bbox (:46-52) is the identity. */
int bh_compute_bbox(bh_context *ctx, double bbox_out[6]);
/* generateMortonCodes (src/morton_keys.cpp:65-98) over the device-resident
 * positions and the bbox of the last bh_compute_bbox.  keys_out may be NULL. */
int bh_compute_keys(bh_context *ctx, uint64_t *keys_out);
/* sortBodiesByMortonKey (include/utility.h:23-52): stable LSD radix sort of
 * the keys, then permutes pos, vel, mass, ids (and keys).  perm_out (may be
 * NULL) receives, for each new position, the body's previous position. */
int bh_sort_bodies(bh_context *ctx, int64_t *perm_out);
/* The caller's own keys (n) in place of bh_compute_keys, e.g. keys made by
 * generateMortonCodes elsewhere; bh_sort_bodies may follow. */
int bh_set_keys(bh_context *ctx, const uint64_t *keys);
/* The caller's global bounding box (the `global_bb` argument of
 * computeAccelerations, include/traversal.h:21-30) in place of
 * bh_compute_bbox. */
int bh_set_bbox(bh_context *ctx, const double bbox[6]);
/* buildOctreeBottomUp alone (merge == 0: centres of mass sum/mass, as the
 * function returns them, src/linear_octree.cpp:95-104) or followed by the
 * single-rank exchange merge (merge != 0, what bh_build_tree does). */
int bh_build_tree_options(bh_context *ctx, int merge);
/* buildOctreeBottomUp (src/linear_octree.cpp:13-107) followed by the
 * single-rank exchangeFullTrees re-merge (src/exchange.cpp:9-29 ->
 * src/linear_octree.cpp:178-204).  Requires sorted keys. */
int bh_build_tree(bh_context *ctx);
/* Sizes of the last tree: n_records = nodes of the reference's uncompressed
 * OctreeMap; n_nodes = nodes of the compressed device octree; n_leaves =
 * distinct keys.  Any pointer may be NULL; with n_records NULL only the
 * counts are read back, otherwise the tree is copied to the host to count
 * the records. */
int bh_tree_info(bh_context *ctx, int64_t *n_records, int64_t *n_nodes, int64_t *n_leaves);
/* The reference's node set (serializeTreeToRecords,
 * src/linear_octree.cpp:169-176, NodeRecord linear_octree.h:60-65) sorted by
 * (depth, prefix): each array holds n_records entries (com: 3 per node). */
int bh_export_tree(bh_context *ctx, uint64_t *prefix, uint8_t *depth, double *mass, double *com);
/* The compressed device tree's nodes (n_nodes of bh_tree_info): the depth
 * and prefix of the reference cell each node stands for (the deepest cell
 * of its single-child chain).  No reference counterpart. */
int bh_tree_slots(bh_context *ctx, uint64_t *prefix, uint8_t *depth);
/* Overrides the mass and centre of mass (com: 3 per node) of every node of
 * the compressed device tree, e.g. with the values of an OctreeMap that the
 * caller changed (the reference's computeAccelerations reads the map it is
 * given).  No reference counterpart. */
int bh_tree_set_slot_values(bh_context *ctx, const double *mass, const double *com);
/* The learned criterion's spread feature per node (n_nodes floats, in the
 * order of bh_tree_slots): sqrt(Q / m) with Q = sum m_i |x_i - com|^2 over
 * the node's bodies, for the far-field masses (bodies with id <
 * BH_NUM_MASSIVE zeroed); 0 for a massless node.  Computes the second-moment
 * pass when the tree in place lacks it.  No reference counterpart. */
int bh_tree_spread(bh_context *ctx, float *spread);
/* createInteractionListForRank (src/exchange.cpp:117-179, include/exchange.h)
 * on the device tree in place: the cells a remote rank whose domain is the
 * union of `boxes` (nboxes x {min.x, min.y, min.z, max.x, max.y, max.z})
 * needs, for the global box `bbox`, opening criterion s^2 >= theta2 * d^2
 * and max_depth (the reference's --max-depth, 21 = full depth).  Writes the
 * NodeRecords (prefix, depth, mass, com: 3 per record) in the tree's node
 * order (the reference returns them in the iteration order of a hash set)
 * and their number to *count_out.  At most one cell per node of
 * bh_tree_info's n_nodes is kept, so that capacity always suffices; a
 * smaller capacity that the count exceeds returns BH_ERR_INVALID_ARGUMENT
 * with *count_out set.  main.cpp exports the local tree of
 * buildOctreeBottomUp, i.e. the tree of bh_build_tree_options(ctx, 0).
 * The arrays may be NULL when the count is 0. */
int bh_let_export(bh_context *ctx, const double *boxes, int64_t nboxes, const double bbox[6], double theta2,
                  int max_depth, int64_t capacity, uint64_t *prefix, uint8_t *depth, double *mass, double *com,
                  int64_t *count_out);
/* buildTreeFromPseudoLeaves (src/linear_octree.cpp:242-322,
 * include/linear_octree.h:85-94) on the device: the map made of m received
 * NodeRecords (records with mass <= 0 or not finite are skipped; depth is
 * clamped to 21 and the prefix masked to it) and all their ancestors, each
 * cell holding the sum of its records' masses and the mass-weighted centre
 * of everything below it (divided by the mass where it exceeds 1e-12).
 * Writes the cells sorted by (depth, prefix) and their number to
 * *count_out; a capacity below the count returns BH_ERR_INVALID_ARGUMENT
 * with *count_out set (sum over records of min(depth, 21) + 1 always
 * suffices).  Duplicate records are summed in input order as in the
 * reference; children are summed in octant order, while the reference sums
 * them in its hash map's iteration order, so cells with several children
 * agree with it to rounding (relative 1e-15).  Uses ctx's device and
 * stream only; the body state is untouched. */
int bh_pseudo_leaf_tree(bh_context *ctx, const uint64_t *prefix, const uint8_t *depth, const double *mass,
                        const double *com, int64_t m, int64_t capacity, uint64_t *out_prefix, uint8_t *out_depth,
                        double *out_mass, double *out_com, int64_t *count_out);
/* computeAccelerationsWithLET (src/traversal.cpp:107-127,
 * include/traversal.h): the m received records become a pseudo-leaf map
 * (as bh_pseudo_leaf_tree), mergeRecordsIntoTree (src/linear_octree.cpp:
 * 178-204) folds it into the local tree in place (built by
 * bh_build_tree_options(ctx, 0) over keys in the global box of bh_set_bbox),
 * and computeAccelerations walks the merged map for the local bodies.
 * The walk repeats the reference's visiting order and IEEE operations, so
 * the result is the reference's on the same merged map; the pseudo-leaf
 * sums (see bh_pseudo_leaf_tree) make it agree with the reference to
 * rounding.  The accelerations replace the context's (acc_out, current
 * body order, may be NULL); the local tree is left as it was. */
int bh_let_accelerations(bh_context *ctx, const uint64_t *prefix, const uint8_t *depth, const double *mass,
                         const double *com, int64_t m, double theta, double G, double soft2, double *acc_out);
/* computeAccelerationsWithRemoteDirectSum (src/traversal.cpp:149-221): the
 * reference's traversal of the local tree (bit-exact, BH_MODE_PLAIN_FP64)
 * plus, per body, a direct sum over the m records (pairs with r^2 <= 1e-12
 * skipped) added to it.  The records are summed in order; the reference's
 * `omp simd` reduction leaves its order to the compiler, so the sum agrees
 * with it to rounding.  prefix and depth are not read (may be NULL). */
int bh_let_direct_accelerations(bh_context *ctx, const uint64_t *prefix, const uint8_t *depth, const double *mass,
                                const double *com, int64_t m, double theta, double G, double soft2,
                                double *acc_out);
/* The bucket boxes of a remote rank's domain as exchangeEssentialTrees
 * builds them (src/exchange.cpp:45-71): bucket prefix p (a key prefix of
 * depth bucket_bits / 3, as update_rank_domains, src/load_balancing.cpp:12-65,
 * stores it) -> min = bbox.min + (i * 2^-d) * span, max = min + span / 2^d
 * per axis.  boxes_out: 6 doubles per prefix.  Host code. */
int bh_let_bucket_boxes(const uint64_t *prefixes, int64_t n, int bucket_bits, const double bbox[6],
                        double *boxes_out);
/* computeAccelerations (src/traversal.cpp:13-103, include/traversal.h:21-30)
 * over the last tree; `mode` is a bh_mode.  acc_out (may be NULL) receives
 * the accelerations in the current body order. */
int bh_compute_accelerations(bh_context *ctx, double theta, double G, double soft2, int mode,
                             double *acc_out);
/* Accepted interactions per body of the last bh_compute_accelerations
 * (summed over the body's accepted nodes). No reference counterpart. */
int bh_interaction_count(bh_context *ctx, int64_t *total_out);
/* Accepted interactions of every body (n int32, current order) in the last
 * bh_compute_accelerations / bh_step.  No reference counterpart. */
int bh_interaction_counts(bh_context *ctx, int32_t *per_body);
/* `nsteps` steps of the `--fc tree` loop of src/main.cpp:191-282 (kick at
 * t > 0, drift, bbox, keys, sort, build, merge, forces, kick).  *t_io is the
 * simulation time, accumulated as t += dt after every step. */
int bh_step(bh_context *ctx, double dt, double theta, double G, int64_t nsteps, int mode, double *t_io);
/* The same loop over a state held on the host, the way the reference's own
 * driver holds it (src/main.cpp:191-282 keeps the bodies in host memory):
 * uploads the n bodies (pos, vel: AoS n*3; mass; ids) and the accelerations
 * of the previous step (acc, n*3, which the first half-kick uses when
 * *t_io > 0), runs nsteps steps, and writes pos, vel, mass, ids and acc back
 * in the new body order.  Equivalent to bh_set_bodies, bh_set_accelerations,
 * bh_step and bh_get_bodies in a row, with one synchronisation instead of
 * five (page-locked host buffers give the fastest copies).  No reference
 * counterpart. */
int bh_step_host(bh_context *ctx, int64_t n, double *pos, double *vel, double *mass, uint64_t *ids, double *acc,
                 double dt, double theta, double G, int64_t nsteps, int mode, double *t_io);

/* ---- measurement (no reference counterpart) -------------------------- */
/* Steps with the kick (all but the first of a run) go through a CUDA graph
 * of the whole step, captured on first use and replayed while the bodies
 * count, mode, dt, theta, G, merge option and direct-body count stay the
 * same (not while profiling).  on = 0 launches every kernel one by one.
 * No reference counterpart. */
int bh_set_step_graphs(bh_context *ctx, int on);
/* Enables (on != 0) or disables CUDA-event timing of the phases of bh_step
 * and clears the accumulated times. */
int bh_set_profiling(bh_context *ctx, int on);
/* Accumulated device time per phase of bh_step since profiling was enabled:
 * ms_out[0] kick+drift+bbox, [1] keys + digit histograms, [2] radix sort,
 * [3] permutation, [4] tree build, [5] forces (+ second half kick);
 * launches_out: kernels this context has enqueued since it was created. */
int bh_phase_times(bh_context *ctx, double ms_out[8], int64_t *launches_out);
/* Sustained FMA throughput of this GPU in TFLOP/s (2 flops per FMA),
 * fp64 != 0 for double, else float: the denominator of the force kernels'
 * roofline, measured in the same process. */
int bh_measure_fma_peak(bh_context *ctx, int fp64, double *tflops_out);

/* ---- diagnostics (no reference counterpart) -------------------------- */
/* FP64 direct sum over all bodies for the bodies at positions targets[k]
 * of the current order; acc_out: ns*3. */
int bh_direct_sum(bh_context *ctx, int64_t ns, const int64_t *targets, double G, double *acc_out);
/* Kinetic energy, potential energy, total angular and linear momentum,
 * out = {E, K, U, Lx, Ly, Lz, Px, Py, Pz}.  theta = 0: U is the exact FP64
 * pair sum (at most 131,072 bodies).  theta > 0: pairs with at least one of
 * the massive bodies (id < BH_NUM_MASSIVE) are exact in FP64 and all other
 * pairs go through the monopoles of the tree of the current positions that
 * the force walk's criterion at theta accepts (any N; the tree is built when
 * none is current, which re-sorts the bodies). */
int bh_invariants(bh_context *ctx, double G, double theta, double out[9]);
/* Checks on the current device of the arithmetic that replaces IEEE
 * divisions and square roots on the hot path, over n seeded inputs;
 * *failures = the number of mismatches.  which = 0: the division-free
 * single-rank merge quotient against RN((0 + RN(m c)) / m); 1: the
 * division-free key quantisation against the IEEE one; 2: the refined
 * reciprocal square root against RN(1 / RN(sqrt x)) (more than 2 ulps
 * apart counts); 3: the division-free centre-of-mass quotient against
 * RN(w / m); 4: the fused r^-3 of the FP64 list form and the direct terms
 * against RN(1 / RN(x RN(sqrt x))) (more than 4 ulps apart counts); 5: the
 * FP32 walk's low part of a centre-of-mass coordinate, formed from the bit
 * patterns, against the FP64 subtraction it replaces.  No reference
 * counterpart. */
int bh_selftest(int which, int64_t n, uint64_t seed, int64_t *failures);

/* ---- learned acceptance (no reference counterpart) ------------------- */
/* The network 8 -> 64 -> 64 -> 1 (ReLU; BF16 weights, FP32 accumulation)
 * predicts log10 of the relative force error of accepting a tree node
 * unopened for a warp's group of bodies.  Parameters are BH_MLP_PARAMS
 * floats: W1[64][8] b1[64] W2[64][64] b2[64] W3[64] b3.  A model's feature
 * scaling is BH_MLP_SCALE floats: per feature mean, 1/std, lowest and
 * highest standardised value seen in training (4 x 8), then the label's mean
 * and std. */
#define BH_MLP_PARAMS 4801
#define BH_MLP_SCALE 34
#define BH_LEARNED_FEATURES 8
/* Loss (mean squared error) and its gradient over n standardised samples
 * X[n][8], targets T[n], computed by the GPU training kernels (for checks). */
int bh_mlp_gradient(const float *params, const float *X, const float *T, int64_t n, float *grad_out,
                    float *loss_out);
/* Trains a network on raw features[n][8] and log10-error labels[n] with
 * Adam (epochs over shuffled mini-batches of `batch`), all on the GPU;
 * returns the parameters, the feature scaling and the last loss of each
 * epoch (loss_out: epochs floats, may be NULL). */
int bh_mlp_train(const float *features, const float *labels, int64_t n, int epochs, int batch, float lr,
                 uint64_t seed, float *params_out, float *scale_out, float *loss_out);

/* A trained model (BH_MLP_PARAMS parameters and BH_MLP_SCALE scaling
 * floats) as a file: an 8-byte tag "BHMLP001", the two counts as uint32,
 * then the floats, all little-endian.  Host functions; BH_ERR_IO on a file
 * that cannot be written or read, BH_ERR_INVALID_ARGUMENT on one that is
 * not such a model. */
int bh_mlp_save(const char *path, const float *params, const float *scale);
int bh_mlp_load(const char *path, float *params_out, float *scale_out);

/* Network outputs (predicted log10 error) for raw feature rows through the
 * same fused mma.sync inference the traversal uses; in_range (may be NULL)
 * flags rows inside the model's training range. */
int bh_mlp_predict(const float *params, const float *scale, const float *features, int64_t n, float *out,
                   int32_t *in_range);
/* Training pairs from the context's bodies (tree built): the FP32 walk with
 * the theta test records every (group, node) the test would not accept for
 * the whole group but theta_max would, with its 8 features
 * (features_out: max_pairs x 8) and its label (labels_out), log10 of the
 * largest relative force error over the group of accepting the node unopened
 * instead of walking its subtree at theta_label.  *n_out pairs are written. */
int bh_learned_collect(bh_context *ctx, double theta, double theta_label, double theta_max, double G,
                       int64_t max_pairs, float *features_out, float *labels_out, int64_t *n_out);
/* Model for BH_MODE_LEARNED.  `budget` is each body's error budget relative
 * to its acceleration: a warp group of 32 bodies starts with an allowance of
 * budget x the smallest of its bodies' direct-term (Sun and planet)
 * accelerations, and every candidate node it accepts unopened pays its
 * predicted error out of it, so the errors a body accepts sum to at most its
 * budget.  A candidate (a node the theta test does not accept for the whole
 * group, side < theta_max d_min) is accepted for the whole group when its
 * predicted error fits both the allowance and its share of it (see
 * bh_learned_set_criterion) and its features are inside the training range;
 * otherwise the theta criterion decides. */
int bh_learned_set_model(bh_context *ctx, const float *params, const float *scale, double budget, double theta_max);
/* Tuning of the criterion (defaults band 0.5, frac 0.25): the analytic error
 * estimate G m s^2 / d_min^4 (s the node's mass spread) decides candidates
 * more than `band` decades below or above the allowance without the network;
 * the network predicts the error of the others.  One candidate takes at most
 * `frac` of the remaining allowance. */
int bh_learned_set_criterion(bh_context *ctx, double band, double frac);
/* Counters of the last BH_MODE_LEARNED traversal: candidates, candidates
 * accepted on the network's prediction, candidates that fell back to theta
 * (features outside the training range), candidates accepted on the
 * analytic estimate. */
int bh_learned_stats(bh_context *ctx, int64_t out[4]);

/* ---- stateless host-buffer entry points ------------------------------ */
/* Each copies its inputs to the device, runs the kernel, copies back.  They
 * use a per-thread default context on device 0. */
int bh_compute_local_bbox(const double *pos, int64_t n, double bbox_out[6]);
int bh_generate_morton_codes(const double *pos, int64_t n, const double bbox[6], uint64_t *keys_out);
int bh_sort_bodies_by_morton_key(int64_t n, uint64_t *keys, double *pos, double *mass, double *vel,
                                 uint64_t *ids);

/* ---- allocation-free sort (no counterpart in the reference) ---------- */
/* For callers that cannot let the library call cudaMalloc: a host code whose
 * device memory belongs to its own pool hands over buffers it already owns,
 * and a time-critical loop cannot take cudaMalloc's implicit device
 * synchronisation or its failure under memory pressure.  Sorts n 63-bit
 * Morton keys already on the device (stable LSD radix sort, the same result
 * as bh_sort_bodies): keys_out receives the sorted keys and perm_out, for
 * each sorted position, the key's input position.  keys_in may equal
 * keys_out.  All three are device pointers; `stream` is a cudaStream_t (NULL
 * for the default stream).  The call allocates nothing: its scratch is a
 * fixed file-scope device array of about 15 MB, held by every GPU that loads
 * the library until the process exits, and n is limited to
 * BH_NOALLOC_MAX_KEYS (larger n returns BH_ERR_CAPACITY).  The first call on
 * a device looks the array's device address up (cudaGetSymbolAddress), so make
 * that first call before any stream capture.  Calls share the array: calls
 * that overlap on the GPU race.  Returns after the sort has finished (it
 * synchronises `stream`). */
#define BH_NOALLOC_MAX_KEYS (1 << 20)
int bh_sort_keys_noalloc(const uint64_t *keys_in, uint64_t *keys_out, uint32_t *perm_out, int64_t n,
                         void *stream);

/* ---- host-side input (no GPU needed) --------------------------------- */
/* convertKeplerToCartesian (src/kepler_to_cartesian.cpp:13-107).
 * el: n*8 = {e, a, i, arg. periapsis, long. asc. node, M, epoch, mu}
 * (radians, AU, days); out: n*6 = {x, y, z, vx, vy, vz}. */
int bh_kepler_to_cartesian(const double *el, int64_t n, double *out);
/* The same conversion for many bodies at once on the current CUDA device
 * (one thread per body; host arrays in and out).  Agrees with
 * bh_kepler_to_cartesian to rounding: the device math functions differ from
 * the host's in their last bits. */
int bh_kepler_to_cartesian_gpu(const double *el, int64_t n, double *out);
/* Seeded synthetic solar system (std::mt19937_64): the Sun (1.989e30 kg at
 * rest at the origin), the 8 planets on circular coplanar orbits, and
 * n - 9 asteroids: an inner belt, a fraction frac_outer in an outer belt
 * (a 30-50 AU) and a fraction frac_trojan in Jupiter's L4/L5 clouds.
 * ids are the row indices.  No reference counterpart (the reference reads
 * CSVs made by its orbital_converter tool). */
int bh_generate_system(uint64_t seed, int64_t n, double frac_outer, double frac_trojan, double *pos,
                       double *vel, double *mass, uint64_t *ids);
/* readCSV (src/io.cpp:16-81): header skipped; columns id,name,class are
 * ignored; mass,pos_x..vel_z parsed; an unparsable line is skipped; ids are
 * the parsed-row counter; at most body_count rows if body_count > 0.
 * Call with pos == NULL to get the row count only. */
int bh_read_csv(const char *path, int64_t body_count, int64_t *n_out, uint64_t *ids, double *mass,
                double *pos, double *vel);
/* readCSV on the current GPU: the same rows, values (bit for bit: std::stod
 * is correctly rounded and so is the device conversion), ids, body_count
 * limit and warnings as bh_read_csv; the file is split and parsed on the
 * device, and the rare fields it cannot decide there (hexadecimal, inf/nan,
 * more than 19 significant digits, results outside the normal range, or
 * within two units of a rounding boundary) are parsed on the host.  With
 * pos == NULL only *n_out is set. */
int bh_read_csv_gpu(const char *path, int64_t body_count, int64_t *n_out, uint64_t *ids, double *mass,
                    double *pos, double *vel);
/* The same, straight into the context's body state (as bh_set_bodies): no
 * host copy of the bodies.  More bodies than the context holds returns
 * BH_ERR_CAPACITY with *n_out set. */
int bh_load_csv(bh_context *ctx, const char *path, int64_t body_count, int64_t *n_out);
/* Writes the reference's state-vector CSV layout (header
 * id,name,class,mass,pos_x,pos_y,pos_z,vel_x,vel_y,vel_z). */
int bh_write_csv(const char *path, int64_t n, const uint64_t *ids, const double *mass, const double *pos,
                 const double *vel);
/* writeSnapshot (src/io.cpp:84-232): one VTK XML PolyData snapshot of n
 * bodies (pos, vel, acc: 3 per body) in the reference's layout and number
 * formatting, for ParaView; rank is the value of the "rank" array (0 for the
 * single-rank path).  As in the reference, n == 0 writes no file.  Host
 * function: no device work. */
int bh_write_vtp(const char *path, int rank, int64_t n, const uint64_t *ids, const double *mass, const double *pos,
                 const double *vel, const double *acc);

#ifdef __cplusplus
}
#endif
#endif /* BH_GPU_H */
