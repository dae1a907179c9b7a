/*
 * zgpu.h -- C ABI of the GB300 walk engine (Walk on Spheres / Walk on Stars fused
 * with the boundary geometric queries they issue every step).
 *
 * Plain C: handles, POD structs, pointers and sizes.  No C++ or torch types cross
 * this boundary.  Every entry point returns a zgpu_status; the message of the most
 * recent failure on the calling thread is available from zgpu_last_error().
 *
 * Each entry point names the interface of rohan-sawhney/zombie it replaces
 * (paths relative to that project).
 */
#ifndef ZGPU_H
#define ZGPU_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define ZGPU_ABI_VERSION 3

/* ------------------------------------------------------------------------- */
/* status codes                                                               */
/* ------------------------------------------------------------------------- */
typedef enum zgpu_status {
    ZGPU_OK = 0,
    ZGPU_ERR_INVALID_ARG = 1,
    ZGPU_ERR_OUT_OF_MEMORY = 2,
    ZGPU_ERR_CUDA = 3,
    ZGPU_ERR_TIMEOUT_BUDGET = 4,       /* a device-side iteration budget ran out */
    ZGPU_ERR_UNSUPPORTED_CALLBACK = 5, /* host std::function callbacks cannot run on the device */
    ZGPU_ERR_UNSUPPORTED = 6,
    ZGPU_ERR_DEVICE_STATE = 7          /* a kernel reported an internal error word */
} zgpu_status;

/* memory space of caller-owned arrays */
enum { ZGPU_MEM_HOST = 0, ZGPU_MEM_DEVICE = 1 };

/* boundary kinds (FcpwDirichlet/Neumann/RobinBoundaryHandler) */
enum { ZGPU_BOUNDARY_ABSORBING = 0, ZGPU_BOUNDARY_NEUMANN = 1, ZGPU_BOUNDARY_ROBIN = 2 };

/* SampleType (point_estimation/common.h:139-143) */
enum { ZGPU_SAMPLE_IN_DOMAIN = 0, ZGPU_SAMPLE_ON_ABSORBING_BOUNDARY = 1, ZGPU_SAMPLE_ON_REFLECTING_BOUNDARY = 2 };

/* EstimationQuantity (point_estimation/common.h:145-149) */
enum { ZGPU_ESTIMATE_SOLUTION = 0, ZGPU_ESTIMATE_SOLUTION_AND_GRADIENT = 1, ZGPU_ESTIMATE_SKIP = 2 };

/* field kinds of the device-evaluable PDE descriptor */
enum { ZGPU_FIELD_ZERO = 0, ZGPU_FIELD_CONSTANT = 1, ZGPU_FIELD_ANALYTIC = 2, ZGPU_FIELD_GRID = 3 };

/* solvers */
enum { ZGPU_SOLVER_WALK_ON_SPHERES = 0, ZGPU_SOLVER_WALK_ON_STARS = 1 };

#define ZGPU_MAX_TERMS 8

/*
 * Closed-form field used as a manufactured solution:
 *   u(x) = sum_k c[k] * exp(a[k].x) * cos(b[k].x + phi[k]) + sum_i q[i] x_i^2 + sum_i l[i] x_i + d
 * Its gradient and Laplacian are closed form, so Dirichlet data g = u, Robin data
 * h = du/dn + kappa u and source f = -Lap(u) + sigma u are evaluated on the device.
 */
typedef struct zgpu_analytic {
    int32_t n_terms;
    float c[ZGPU_MAX_TERMS];
    float a[ZGPU_MAX_TERMS][3];
    float b[ZGPU_MAX_TERMS][3];
    float phi[ZGPU_MAX_TERMS];
    float q[3];
    float l[3];
    float d;
} zgpu_analytic;

/*
 * A dense grid field (DenseGrid<float, 1, DIM>, utils/dense_grid.h) over the box
 * [grid_min, grid_max], cell-centred samples, row-major with the last axis fastest
 * (value of cell (i, j[, k]) at (i * shape[1] + j)[* shape[2] + k]).  Lookups clamp to the
 * grid: nearest cell, or (enable_interpolation) bi/trilinear between cell centres with the
 * blend fractions clamped to [0, 1] (dense_grid.h:264-355).  values_aligned is the grid
 * returned for returnBoundaryNormalAlignedValue = true (getDenseGridCallback2/4,
 * dense_grid.h:442-560); NULL -> values.
 */
typedef struct zgpu_grid {
    const float* values;          /* device or host pointer, see zgpu_pde.memory */
    const float* values_aligned;
    int32_t shape[3];
    float grid_min[3];
    float grid_max[3];
    int32_t enable_interpolation;
} zgpu_grid;

/*
 * Device-evaluable replacement for PDE<T,DIM> (core/pde.h:19-45), whose members are
 * host std::functions.  Each field is ZERO, CONSTANT (value), ANALYTIC (derived from
 * `solution`) or GRID.  The *_aligned values are those returned when the reference
 * passes returnBoundaryNormalAlignedValue = true (double-sided problems).
 */
typedef struct zgpu_pde {
    float absorption_coeff;                  /* sigma >= 0 in  -Lap u + sigma u = f */
    int32_t is_source_constant;
    int32_t are_robin_conditions_pure_neumann;
    int32_t are_robin_coeffs_nonnegative;
    zgpu_analytic solution;
    int32_t source_kind;       float source_value;
    int32_t dirichlet_kind;    float dirichlet_value;    float dirichlet_value_aligned;
    int32_t robin_kind;        float robin_value;        float robin_value_aligned;
    int32_t robin_coeff_kind;  float robin_coeff_value;  float robin_coeff_value_aligned;
    zgpu_grid source_grid;
    zgpu_grid dirichlet_grid;
    zgpu_grid robin_grid;
    zgpu_grid robin_coeff_grid;
    int32_t memory;            /* memory space of the grid value arrays (host arrays are copied
                                  to the device by each solve) */
} zgpu_pde;

/* WalkSettings (point_estimation/common.h:19-91): same fields, same order. */
typedef struct zgpu_walk_settings {
    float epsilon_shell_for_absorbing_boundary;
    float epsilon_shell_for_reflecting_boundary;
    float silhouette_precision;
    float russian_roulette_threshold;
    float splitting_threshold;
    int32_t max_walk_length;
    int32_t steps_before_applying_tikhonov;
    int32_t steps_before_using_maximal_spheres;
    int32_t solve_double_sided;
    int32_t use_gradient_control_variates;
    int32_t use_gradient_antithetic_variates;
    int32_t use_cosine_sampling_for_derivatives;
    int32_t ignore_absorbing_boundary_contribution;
    int32_t ignore_reflecting_boundary_contribution;
    int32_t ignore_source_contribution;
    int32_t print_logs;
} zgpu_walk_settings;

/*
 * SamplePoint (point_estimation/common.h:151-195) as structure of arrays.
 * pt/normal are [n*dim] floats.  seed[i] replaces the per-point pcg32 member: walk w
 * of point i draws from pcg32(seed[i], stream = w + statistics n[i]).
 * first_sphere_radius is read and written (WoSt precomputes it on the first call).
 * Optional arrays may be NULL (normal -> 0, type -> IN_DOMAIN, dist_to_reflecting -> inf,
 * estimate_normal_aligned -> 0, estimation_quantity -> SOLUTION).
 */
typedef struct zgpu_sample_points {
    int64_t n;
    int32_t memory;
    const float* pt;
    const float* normal;
    const int32_t* type;
    const int32_t* estimation_quantity;
    const float* dist_to_absorbing;
    const float* dist_to_reflecting;
    const int32_t* n_walks;
    const uint64_t* seed;
    float* first_sphere_radius;
    const int32_t* estimate_normal_aligned;
    const int32_t* scene_id;   /* batched many-solve: index into the scene table, NULL -> 0 */
    const float* direction_for_derivative;  /* [n*dim] SamplePoint::directionForDerivative
                                               (common.h:185), NULL -> (1, 0[, 0]) */
} zgpu_sample_points;

/*
 * SampleStatistics (point_estimation/common.h:200-395) as structure of arrays,
 * accumulated across calls (progressive estimation, as the reference): every solve
 * merges its walks into these arrays with the parallel Welford merge of
 * SampleStatistics::merge (common.h:268-310), in FP64.
 * gradient_mean/gradient_m2 are [n*dim] and may be NULL when no point asks for gradients.
 * total_first_source_contribution and total_derivative_contribution are the running sums
 * behind getMeanFirstSourceContribution and getEstimatedDerivative (common.h:346-355), added
 * to by gradient walks; either may be NULL (the source control variate is then 0).
 */
typedef struct zgpu_sample_statistics {
    int32_t memory;
    double* solution_mean;
    double* solution_m2;
    int32_t* n_solution_estimates;
    int64_t* total_walk_length;
    int64_t* total_splits;
    double* gradient_mean;
    double* gradient_m2;
    int32_t* n_gradient_estimates;
    double* total_first_source_contribution;
    double* total_derivative_contribution;
} zgpu_sample_statistics;

/* launch and engine options that have no counterpart in the reference */
/* zgpu_solve_options.schedule */
#define ZGPU_SCHEDULE_AUTO 0
#define ZGPU_SCHEDULE_PERSISTENT 1
#define ZGPU_SCHEDULE_WAVEFRONT 2

typedef struct zgpu_solve_options {
    int32_t block_size;        /* 0 -> autotuned / default */
    int32_t blocks_per_sm;     /* 0 -> occupancy-derived */
    int32_t use_graph;         /* capture prepare+walk+finalize in a CUDA graph and replay (the
                                  wavefront schedule: chunks of its iterations) */
    int32_t query_mode;        /* closest-point queries of Walk on Spheres and Robin star radii of
                                  Walk on Stars: 0 auto, 1 one lane per query, 2 the whole warp
                                  per query (large scenes) */
    int64_t step_budget;       /* per-walk-state cap on device loop iterations (0: none beyond
                                  max_walk_length); a walk that reaches it is dropped and the
                                  solve returns ZGPU_ERR_TIMEOUT_BUDGET */
    int32_t bvh_width;         /* 0 / 4: the boundaries' own trees; 8: an 8-wide tree of a 3D
                                  absorbing boundary built on the host (built once, on first use,
                                  from the boundary's copy of its mesh) */
    int32_t schedule;          /* walk loop: 0 auto, 1 the persistent kernel (one lane per walk
                                  from start to end), 2 the sorted wavefront (walk states in device
                                  memory, sorted by position every step; solutions only, no cache
                                  or warp-wide queries, non-negative Robin coefficients, splitting
                                  threshold >= 2; batched solves too; with use_graph its iterations
                                  replay from a captured graph).  Auto picks the wavefront for the
                                  2D Walk on Stars solves it can serve. */
} zgpu_solve_options;

/* counters returned by a solve */
typedef struct zgpu_solve_report {
    uint64_t total_steps;      /* executed walk-loop iterations (the walk-steps/s numerator) */
    uint64_t total_walks;
    uint64_t escaped_walks;
    uint64_t exceeded_walks;
    uint64_t rr_terminated;
    float kernel_ms;           /* CUDA-event time of the walk kernel */
    float total_ms;            /* CUDA-event time of prepare + walk + finalize */
    uint32_t error_word;       /* nonzero: device-side internal error (stack overflow, budget) */
    uint64_t cache_terminated; /* walks ended through the neural cache (zgpu_solve_cached) */
} zgpu_solve_report;

typedef struct zgpu_context zgpu_context;
typedef struct zgpu_boundary zgpu_boundary;

/*
 * GeometricQueries<DIM> (core/geometric_queries.h:58-124) populated by
 * populateGeometricQueriesFor{Dirichlet,Neumann,Robin}Boundary
 * (utils/fcpw_geometric_queries.h:1062-1389): the std::function members become the
 * device queries of the two boundary handles.  Either handle may be NULL (empty part).
 */
typedef struct zgpu_geometric_queries {
    int32_t dim;
    int32_t domain_is_watertight;
    float domain_min[3];
    float domain_max[3];
    zgpu_boundary* absorbing;
    zgpu_boundary* reflecting;
} zgpu_geometric_queries;

/* ---------------------------- context ------------------------------------ */
int zgpu_abi_version(void);
const char* zgpu_last_error(void);
/* creates a context (CUDA stream + cached scratch) on `device` */
int zgpu_context_create(int device, zgpu_context** out);
int zgpu_context_destroy(zgpu_context* ctx);
int zgpu_context_synchronize(zgpu_context* ctx);
/* the CUDA stream (cudaStream_t) every kernel of this context is launched on */
void* zgpu_context_stream(zgpu_context* ctx);

/* ---------------------------- boundaries --------------------------------- */
/*
 * Builds a boundary acceleration structure on the device.  Replaces
 * FcpwDirichletBoundaryHandler::buildAccelerationStructure (utils/fcpw_geometric_queries.h:84-88),
 * FcpwNeumannBoundaryHandler::buildAccelerationStructure (:100-105, silhouettes from
 * computeSilhouettes :631) and FcpwRobinBoundaryHandler::buildAccelerationStructure
 * (:117-124, adjacency :745-799 / :892-973, ReflectanceBvh reflectance_boundary_bvh/bvh.h).
 * positions: [n_vertices*dim] host floats; indices: [n_prims*dim] host ints.
 * min/max_robin_coeff: [n_prims] (ROBIN only, else NULL).
 * solve_double_sided/silhouette_precision feed getIgnoreCandidateSilhouetteCallback (:1029-1038).
 * bvh_width: 4 or 8 (0 -> 4); 8-wide trees are built for 3D absorbing boundaries only
 * (other boundaries return ZGPU_ERR_UNSUPPORTED for 8), and they do not serve
 * zgpu_query_sample_boundary.
 */
int zgpu_boundary_create(zgpu_context* ctx, int dim, const float* positions, int n_vertices,
                         const int* indices, int n_prims, int kind,
                         const float* min_robin_coeff, const float* max_robin_coeff,
                         int solve_double_sided, float silhouette_precision, int bvh_width,
                         zgpu_boundary** out);
int zgpu_boundary_destroy(zgpu_boundary* b);
/* FcpwRobinBoundaryHandler::updateCoefficientValues (utils/fcpw_geometric_queries.h:126-128) */
int zgpu_boundary_update_robin_coefficients(zgpu_boundary* b, const float* min_robin_coeff,
                                            const float* max_robin_coeff);
/* statistics of the built tree: nodes, depth, bytes (for the roofline bookkeeping) */
int zgpu_boundary_info(zgpu_boundary* b, int64_t* n_nodes, int32_t* depth, int64_t* node_bytes,
                       int64_t* prim_bytes);
/* Aggregate::signedVolume (used by computeAbsorbing/ReflectingBoundarySignedVolume) */
int zgpu_boundary_signed_volume(zgpu_boundary* b, float* out);

/* ---------------------- batched geometric queries ------------------------- */
/* All arrays live in `memory`; n queries; vectors are [n*dim].                */

/*
 * How the batched queries below traverse the tree (no counterpart in the reference, whose
 * queries run one CPU thread per query): ZGPU_QUERY_MODE_AUTO / _LANE answer each query on one
 * GPU lane; ZGPU_QUERY_MODE_WARP answers closest-point queries, and star-radius queries of
 * Robin boundaries, with a whole warp per query (the traversal the walk kernel uses on large
 * scenes with zgpu_solve_options.query_mode = 2).  Both modes return the same primitive for
 * every closest-point query; Robin radii agree up to node bounds met in another order.
 */
#define ZGPU_QUERY_MODE_AUTO 0
#define ZGPU_QUERY_MODE_LANE 1
#define ZGPU_QUERY_MODE_WARP 2
int zgpu_boundary_set_query_mode(zgpu_boundary* b, int mode);

/* computeDistToAbsorbingBoundary / projectToAbsorbingBoundary
 * (utils/fcpw_geometric_queries.h:1069-1096; reflecting twins :1150-1177):
 * closest point, its normal, (signed) distance and the caller's primitive index. */
int zgpu_query_closest_point(zgpu_boundary* b, int64_t n, const float* x, int compute_signed,
                             float* out_pt, float* out_normal, float* out_dist, int32_t* out_prim,
                             int memory);
/* intersectAbsorbingBoundary / intersectReflectingBoundary (:1097-1115, :1178-1196):
 * first hit within t_max; origins on the boundary are offset along -normal. */
int zgpu_query_intersect(zgpu_boundary* b, int64_t n, const float* origin, const float* normal,
                         const float* dir, const float* t_max, const int32_t* on_boundary,
                         int32_t* out_hit, float* out_pt, float* out_normal, float* out_dist,
                         int32_t* out_prim, int memory);
/* intersect...AllHits (:1116-1136, :1197-1217): number of hits within t_max */
int zgpu_query_count_hits(zgpu_boundary* b, int64_t n, const float* origin, const float* dir,
                          const float* t_max, int32_t* out_count, int memory);
/* computeStarRadiusForReflectingBoundary (Neumann :1249-1270, Robin :1272-1291) */
int zgpu_query_star_radius(zgpu_boundary* b, int64_t n, const float* x, const float* min_radius,
                           const float* max_radius, float silhouette_precision,
                           const int32_t* flip_normal_orientation, float* out_radius, int memory);
/* intersectsWithReflectingBoundary (:1218-1226): 1 when the segment xi->xj is occluded */
int zgpu_query_occluded(zgpu_boundary* b, int64_t n, const float* xi, const float* xj,
                        const float* ni, const float* nj, const int32_t* offset_i,
                        const int32_t* offset_j, int32_t* out_occluded, int memory);
/* sampleReflectingBoundary (:1227-1242): a boundary point inside the ball with its pdf */
int zgpu_query_sample_boundary(zgpu_boundary* b, int64_t n, const float* x, const float* radius,
                               const float* rand_nums, int32_t* out_found, float* out_pt,
                               float* out_normal, float* out_pdf, int memory);

/*
 * zgpu_boundary_create with everything built on the GPU (no counterpart in the reference,
 * which builds on the CPU): a linear BVH over Morton codes of the primitive centres,
 * collapsed to the same 4-wide node layout; for reflecting boundaries also the face
 * adjacency, silhouette flags, normal cones (merged bottom-up: possibly wider than the host
 * builder's, never narrower), Robin coefficient ranges and the silhouette-candidate tree.
 * positions / indices / min_robin / max_robin live in host or device memory (`memory`).
 * Queries answer as on a host-built tree; a tree deeper than the traversal stack returns
 * ZGPU_ERR_UNSUPPORTED.
 */
int zgpu_boundary_create_on_device(zgpu_context* ctx, int dim, const float* positions, int n_vertices,
                                   const int* indices, int n_prims, int kind, const float* min_robin,
                                   const float* max_robin, int solve_double_sided, float silhouette_precision,
                                   int memory, zgpu_boundary** out);

/* ------------------------------- solve ----------------------------------- */
/*
 * WalkOnSpheres<T,DIM>::solve (point_estimation/walk_on_spheres.h:38-44, batch over points
 * :132-168) and WalkOnStars<T,DIM>::solve (point_estimation/walk_on_stars.h:40-46, :151-187).
 * Runs every walk of every point, in one persistent kernel or (options->schedule; the
 * default for 2D Walk on Stars) as a sorted wavefront of walk records, and merges the walk
 * estimates into `stats`.  options/report may be NULL.
 */
int zgpu_solve(zgpu_context* ctx, int solver, const zgpu_geometric_queries* queries,
               const zgpu_pde* pde, const zgpu_walk_settings* settings,
               const zgpu_sample_points* points, zgpu_sample_statistics* stats,
               const zgpu_solve_options* options, zgpu_solve_report* report);

/* Kernel launches issued by the last solve on `ctx` (zgpu_solve, zgpu_solve_batched,
 * zgpu_solve_cached): prepare, the walk-id scan, the walk kernel or the wavefront's
 * iterations (6 launches each, 5 for Walk on Spheres) and its drain, the cache pass and
 * finalize.  No counterpart in the reference. */
int zgpu_last_solve_launches(zgpu_context* ctx, int64_t* launches);

/*
 * Batched many-solve: `n_scenes` independent problems of one dimension (2D or 3D) in one
 * launch.  points->scene_id selects the row of queries/pdes/settings for every point; each
 * point runs the walks it runs in a single-scene solve.
 */
int zgpu_solve_batched(zgpu_context* ctx, int solver, int n_scenes,
                       const zgpu_geometric_queries* queries, const zgpu_pde* pdes,
                       const zgpu_walk_settings* settings, const zgpu_sample_points* points,
                       zgpu_sample_statistics* stats, const zgpu_solve_options* options,
                       zgpu_solve_report* report);

/*
 * Autotuner (no counterpart in the reference): times launch configurations (block size
 * 32/64/128 x blocks per SM auto/2/4, the query mode for Walk on Spheres and for Walk on
 * Stars on a Robin boundary, and the BVH node width 4 / 8 of a 3D absorbing boundary) on a
 * stride sample of `sample_points` points with `sample_walks` walks each, and writes the
 * fastest into `out_options`.  Results are cached in the context per scene signature
 * (dimension, solver, log2 primitive counts, reflecting kind, screening); a cached answer
 * returns with *best_steps_per_s = -1.  There is no walks-per-thread knob: the persistent
 * walk kernel refills each lane from a global walk counter whenever its walk ends, so a lane
 * runs as many walks as the load demands, and the wavefront keeps a fixed pool of 2^23 walks
 * in flight (about 43 per resident thread).  The candidates run on the persistent kernel (the
 * sample is too small to measure the wavefront schedule fairly) and the options returned keep the
 * automatic schedule.
 */
int zgpu_autotune(zgpu_context* ctx, int solver, const zgpu_geometric_queries* queries, const zgpu_pde* pde,
                  const zgpu_walk_settings* settings, const zgpu_sample_points* points, int32_t sample_points,
                  int32_t sample_walks, zgpu_solve_options* out_options, float* best_steps_per_s);

/* ------------------------- allocation-free solve -------------------------- */
/*
 * zgpu_solve_static: a variant of zgpu_solve that allocates nothing.  No counterpart in the
 * reference; it exists for callers that must not allocate device memory, such as a plug-in
 * whose host application owns the GPU memory budget, or a real-time loop that forbids
 * cudaMalloc after start-up.  The caller passes inputs and outputs in device memory and the
 * CUDA stream to run on (cudaStream_t, NULL = legacy default stream), with that stream's
 * device current.  All scratch (walk prefix, per-point flags and FP64 accumulators,
 * counters) lives in one file-scope __device__ array of ZGPU_STATIC_SCRATCH_BYTES that every
 * GPU loading the library holds until process exit.
 * Limits: points->n <= ZGPU_STATIC_MAX_POINTS; points and statistics in ZGPU_MEM_DEVICE;
 * no walk splitting (splitting_threshold must be FLT_MAX).  Larger inputs are rejected with
 * ZGPU_ERR_INVALID_ARG.  Solution only, single scene: gradient statistics arrays or a
 * scene_id array are rejected with ZGPU_ERR_UNSUPPORTED.  The first call on a device looks
 * up the array's device address and keeps it until exit (it assumes the device's primary
 * context is not reset meanwhile); make that first call before any stream capture.  Every call shares the one array and
 * clears what must start at zero: calls that overlap on the GPU (two streams, two host
 * threads) race and must be serialised by the caller.  The call returns after the stream
 * has drained (it reads back the counters for the report and the error word).
 */
#define ZGPU_STATIC_MAX_POINTS 65536
#define ZGPU_STATIC_SCRATCH_BYTES (4u << 20)
int zgpu_solve_static(void* stream, int solver, const zgpu_geometric_queries* queries, const zgpu_pde* pde,
                      const zgpu_walk_settings* settings, const zgpu_sample_points* points,
                      zgpu_sample_statistics* stats, zgpu_solve_report* report);

/* ------------------------------ neural cache ------------------------------ */
/*
 * A learned cache of the solution: a multiresolution hash-grid encoding (n_levels levels of
 * 2 FP16 features, 2^log2_table_size entries per level, resolutions growing geometrically
 * from base_resolution to max_resolution over the domain box) feeding a 32-64-64-1 ReLU MLP
 * with BF16 weights evaluated on the tensor cores (FP32 accumulation).  No counterpart in
 * the reference.  It is trained online on walk estimates (zgpu_cache_train, Adam on the
 * mean squared error), and zgpu_solve_cached ends a walk at its first position after the
 * first step that lies at least min_distance from the boundary, paying
 * throughput * cache(x) there.  The plain walk (zgpu_solve) stays the fallback.
 */
typedef struct zgpu_cache zgpu_cache;

typedef struct zgpu_cache_config {
    int32_t dim;                 /* 2 or 3 */
    int32_t n_levels;            /* 1..16 (encoding width 32; unused levels encode 0) */
    int32_t log2_table_size;     /* 8..24 */
    float base_resolution;       /* coarsest grid resolution (>= 1) */
    float max_resolution;        /* finest grid resolution */
    float domain_min[3];         /* box mapped to [0,1]^dim before encoding */
    float domain_max[3];
    float learning_rate_grid;    /* Adam step of the table */
    float learning_rate_mlp;     /* Adam step of the network */
    float beta1, beta2, epsilon; /* Adam moments */
    uint64_t seed;               /* initialisation */
} zgpu_cache_config;

int zgpu_cache_create(zgpu_context* ctx, const zgpu_cache_config* config, zgpu_cache** out);
int zgpu_cache_destroy(zgpu_cache* cache);
/* offsets[8] into the flat FP32 parameter vector: table [levels][T][2], W1 [64][32], b1 [64],
 * W2 [64][64], b2 [64], w3 [64], b3, total */
int zgpu_cache_layout(const zgpu_cache* cache, int64_t* offsets);
/* the integer resolution of each level (n_levels floats) */
int zgpu_cache_resolutions(const zgpu_cache* cache, float* res);
/* changes the Adam step sizes of later zgpu_cache_train calls (a decay schedule) */
int zgpu_cache_set_learning_rates(zgpu_cache* cache, float learning_rate_grid, float learning_rate_mlp);
int zgpu_cache_get_parameters(zgpu_cache* cache, float* out_params);
int zgpu_cache_set_parameters(zgpu_cache* cache, const float* params);
/* `steps` Adam steps on batches of batch_size consecutive (wrapping) points of the training
 * set (pass it in random order); mean_loss (may be NULL) = mean squared error over them */
int zgpu_cache_train(zgpu_cache* cache, int64_t n, const float* x, const float* target, int memory,
                     int32_t steps, int32_t batch_size, float* mean_loss);
/* gradient of the mean squared error over all n points (no update); grads laid out as the
 * parameters */
int zgpu_cache_gradients(zgpu_cache* cache, int64_t n, const float* x, const float* target, int memory,
                         float* grads, double* loss);
int zgpu_cache_evaluate(zgpu_cache* cache, int64_t n, const float* x, float* y, int memory);
/* the FP32 hash-grid encoding of each point, enc [n][32] (for inspection and tests) */
int zgpu_cache_encode(zgpu_cache* cache, int64_t n, const float* x, float* enc, int memory);

/*
 * zgpu_solve with early walk termination through the cache: once a walk has taken a step and
 * its position lies at least min_distance from the absorbing boundary (and, for Walk on
 * Stars, from the reflecting boundary, off it), the walk ends and its estimate is the
 * contributions gathered so far plus throughput * cache(x).  Walk splitting is not supported
 * (splitting_threshold must be FLT_MAX).  report->rr_terminated etc. count as in zgpu_solve;
 * cache-terminated walks are reported in report->total_walks like the others.
 */
int zgpu_solve_cached(zgpu_context* ctx, int solver, const zgpu_geometric_queries* queries,
                      const zgpu_pde* pde, const zgpu_walk_settings* settings,
                      const zgpu_sample_points* points, zgpu_sample_statistics* stats,
                      const zgpu_solve_options* options, zgpu_cache* cache, float min_distance,
                      zgpu_solve_report* report);

/* ------------------------------ PDE fields -------------------------------- */
/*
 * The PDE's fields at n points as the walks read them: source(x), dirichlet(x, aligned),
 * robin(x, n, aligned), robinCoeff(x, n, aligned) (core/pde.h:29-41).  normal and aligned may
 * be NULL (zero normal, not aligned); any output may be NULL.  All arrays in `memory`.
 */
int zgpu_pde_evaluate(zgpu_context* ctx, int dim, const zgpu_pde* pde, int64_t n, const float* x,
                      const float* normal, const int32_t* aligned, int memory, float* out_source,
                      float* out_dirichlet, float* out_robin, float* out_robin_coeff);

/* ------------------------- boundary value caching -------------------------- */
/*
 * Boundary Value Caching (variance_reduction/boundary_value_caching.h).  A cache is a set of
 * SamplePoints with the members the splat reads: position, normal, pdf, type
 * (ZGPU_SAMPLE_ON_ABSORBING_BOUNDARY / ON_REFLECTING_BOUNDARY: boundary samples;
 * ZGPU_SAMPLE_IN_DOMAIN: source samples), estimate_normal_aligned, and the estimated
 * solution, normalDerivative, contribution (Robin data or source value) and robinCoeff.
 */
typedef struct zgpu_bvc_samples {
    int64_t n;
    const float* pt;                  /* [n*dim] */
    const float* normal;              /* [n*dim] */
    const float* pdf;
    const int32_t* type;
    const int32_t* estimate_normal_aligned;   /* NULL -> 0 */
    const float* solution;
    const float* normal_derivative;
    const float* contribution;
    const float* robin_coeff;         /* NULL -> 0 */
} zgpu_bvc_samples;

/* ZGPU_BVC_* : the five statistics of an EvaluationPoint (boundary_value_caching.h:19-56) */
enum { ZGPU_BVC_ABSORBING = 0, ZGPU_BVC_ABSORBING_ALIGNED = 1, ZGPU_BVC_REFLECTING = 2,
       ZGPU_BVC_REFLECTING_ALIGNED = 3, ZGPU_BVC_SOURCE = 4, ZGPU_BVC_GROUPS = 5 };

/*
 * EvaluationPoints as structure of arrays; each holds five SampleStatistics (solution and
 * gradient moments, FP64), indexed [point][group] and [point][group][dim].  The estimated
 * solution of a point is the sum of its five means (EvaluationPoint::getEstimatedSolution).
 */
typedef struct zgpu_bvc_eval_points {
    int64_t n;
    const float* pt;                  /* [n*dim] */
    const int32_t* type;              /* NULL -> IN_DOMAIN */
    const float* dist_to_absorbing;
    const float* dist_to_reflecting;  /* NULL -> +inf */
    double* mean;                     /* [n*5] */
    double* m2;                       /* [n*5] */
    int32_t* count;                   /* [n*5] */
    double* gradient_mean;            /* [n*5*dim] */
    double* gradient_m2;              /* [n*5*dim], may be NULL */
} zgpu_bvc_eval_points;

/*
 * BoundaryValueCaching::splat (boundary_value_caching.h:408-425, :652-811): every sample of
 * the cache splats its free-space Green's function estimate (harmonic, or Yukawa when the
 * PDE's absorption coefficient is > 0) onto every evaluation point at least the cutoff
 * distances from the boundaries; statistics merge with what the points already hold.
 */
int zgpu_bvc_splat(zgpu_context* ctx, int dim, const zgpu_pde* pde, const zgpu_bvc_samples* samples,
                   float radius_clamp, float kernel_regularization, float robin_coeff_cutoff_for_normal_derivative,
                   float cutoff_dist_to_absorbing_boundary, float cutoff_dist_to_reflecting_boundary,
                   zgpu_bvc_eval_points* eval_points, int memory);

/* ------------------------- reverse walk on stars --------------------------- */
/*
 * Reverse Walk on Stars (point_estimation/reverse_walk_on_stars.h, variance_reduction/
 * reverse_walk_solver.h): one walk per sample point, started at the sample, that splats the
 * sample's contribution (source value, Dirichlet value of an absorbing sample offset into the
 * domain, or Robin data) onto every evaluation point inside each step's star-shaped ball
 * and visible from the walk position, weighted by the ball's Green's function.
 */
typedef struct zgpu_rws_samples {
    int64_t n;
    const float* pt;                  /* [n*dim] */
    const float* normal;              /* [n*dim] */
    const int32_t* type;              /* ZGPU_SAMPLE_* */
    const int32_t* estimate_normal_aligned;   /* NULL -> 0 */
    const float* pdf;
    const float* contribution;        /* SamplePoint::contribution set by the caller */
    const float* dist_to_absorbing;
    const uint64_t* seed;             /* walk of sample i: pcg32(seed[i], stream) */
} zgpu_rws_samples;

/* ZGPU_RWS_* : the running sums of an rws::EvaluationPoint (reverse_walk_solver.h:19-45) */
enum { ZGPU_RWS_ABSORBING = 0, ZGPU_RWS_ABSORBING_ALIGNED = 1, ZGPU_RWS_REFLECTING = 2,
       ZGPU_RWS_REFLECTING_ALIGNED = 3, ZGPU_RWS_SOURCE = 4, ZGPU_RWS_POISSON_KERNEL = 5, ZGPU_RWS_TOTALS = 6 };

typedef struct zgpu_rws_eval_points {
    int64_t n;
    const float* pt;                  /* [n*dim] */
    const float* normal;              /* [n*dim], NULL -> 0 */
    const int32_t* type;              /* NULL -> IN_DOMAIN; absorbing points are not splatted */
    double* totals;                   /* [n*6], added to */
} zgpu_rws_eval_points;

/*
 * One call of ReverseWalkOnStars::solve over all samples (one walk each, pcg32 stream
 * `stream`), splatting into eval_points->totals.  Absorbing samples' splats are divided by
 * normal_offset_for_absorbing_boundary; the Poisson-kernel total (self-normalisation) is kept
 * when the domain is watertight, the PDE unscreened and the reflecting boundary (if any) pure
 * Neumann.  report->total_steps counts walk steps, report->total_walks the walks.
 */
int zgpu_rws_solve(zgpu_context* ctx, const zgpu_geometric_queries* queries, const zgpu_pde* pde,
                   const zgpu_walk_settings* settings, const zgpu_rws_samples* samples,
                   float normal_offset_for_absorbing_boundary, float radius_clamp, float kernel_regularization,
                   uint64_t stream, zgpu_rws_eval_points* eval_points, int memory, zgpu_solve_report* report);

#ifdef __cplusplus
}
#endif
#endif /* ZGPU_H */
