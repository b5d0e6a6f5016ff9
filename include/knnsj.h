/*
 * knnsj.h -- C ABI of the GB300-native exact k-nearest-neighbour self-join.
 *
 * Drop-in boundary for the GPU-only kNN self-join of
 * mgowanlock/hybrid_k_nearest_neighbor_self_join.  Every entry point takes
 * plain pointers and sizes; no CUDA, C++ or Python type appears here.
 *
 * Result convention (shared by every entry point, as in the reference's
 * KNNJoinPy, main.cu:514 and storeNeighborTableForkNNOnTheFly,
 * GPU.cu:3610-3704): for N points and a user k, the caller owns
 *   int32_t ids[N * (k+1)]   and   DTYPE dists[N * (k+1)]
 * and row q (offset q*(k+1)) receives the k+1 nearest points of point q --
 * the point itself included -- in ascending Euclidean distance.  Distances
 * are sqrt of the squared distance summed in DTYPE with one fused
 * multiply-add per dimension, over the dimensions reordered by decreasing
 * sampled variance (main.cu:2521-2615, kernel.cu:116-161).  Equal distances
 * are ordered by point id.
 *
 * Threading: one join at a time per process; calls from several host
 * threads are serialised internally.
 */
#ifndef KNNSJ_H
#define KNNSJ_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define KNNSJ_VERSION_MAJOR 1
#define KNNSJ_VERSION_MINOR 0

/* Status codes.  The reference returns nothing and prints its errors
 * (main.cu:141-146, 338-342, GPU.cu:150-152); every entry point here
 * reports one of these instead. */
typedef enum {
  KNNSJ_OK = 0,
  KNNSJ_ERR_INVALID_ARGUMENT = 1, /* null pointer, n == 0, d == 0, d > 256, ... */
  KNNSJ_ERR_DIM_MISMATCH = 2,     /* NDIM != GPUNUMDIM of a fixed build (main.cu:141) */
  KNNSJ_ERR_K_TOO_LARGE = 3,      /* k+1 > N: the reference loops forever (main.cu:312) */
  KNNSJ_ERR_NONFINITE_INPUT = 4,  /* NaN or infinite coordinate */
  KNNSJ_ERR_TOO_MANY_POINTS = 5,  /* N >= 2^31: ids are int32 */
  KNNSJ_ERR_NO_CONVERGENCE = 6,   /* iteration cap reached */
  KNNSJ_ERR_CUDA = 7,             /* CUDA runtime error */
  KNNSJ_ERR_OUT_OF_MEMORY = 8,
  KNNSJ_ERR_NO_DEVICE = 9,
  KNNSJ_ERR_UNSUPPORTED = 10,     /* e.g. NUMINDEXEDDIM > 8, k+1 > 16352 (float) or 8160 (double) */
  KNNSJ_ERR_IO = 11,              /* file could not be read or written */
  KNNSJ_ERR_EXCEEDS_FIXED_SCRATCH = 12 /* knnsj_selfjoin_device_noalloc: problem too large */
} knnsj_status;

typedef enum { KNNSJ_F32 = 0, KNNSJ_F64 = 1 } knnsj_dtype;

/* How each query's starting radius is chosen. */
typedef enum {
  KNNSJ_RADIUS_BETA = 0,   /* reference rule: eps0 from BETA for every query */
  KNNSJ_RADIUS_LEARNED = 1 /* learned per-query starting radius (new; no
                              reference counterpart); acceptance stays exact */
} knnsj_radius_mode;

/* Options.  Zero-initialise, set struct_size = sizeof(knnsj_options), then
 * override fields.  A zero / negative value selects the default, which is the
 * reference's params.h value or the environment override named beside it. */
typedef struct {
  uint32_t struct_size;
  int32_t num_indexed_dims; /* NUMINDEXEDDIM (params.h:9); default min(d, 6)
                               [KNNSJ_NUMINDEXEDDIM]; at most 8 */
  double beta;              /* BETA (params.h:58); < 0 -> 0.05 [KNNSJ_BETA] */
  int32_t no_reorder;       /* 1 disables REORDER (params.h:37) */
  int32_t radius_mode;      /* knnsj_radius_mode */
  int32_t max_iterations;   /* radius re-attempts cap; 0 -> automatic */
  int32_t device;           /* CUDA device ordinal; < 0 -> current device */
  int32_t verbose;          /* 1 prints phase timings on stderr [KNNSJ_VERBOSE] */
  double radius_offset;     /* KNNSJ_RADIUS_LEARNED: added to the predicted
                               log(radius / eps0); 0 = the model as trained */
  int32_t device_table_mb;  /* host-pointer calls with pageable outputs: the
                               largest device result table (MB) before the
                               outputs are registered with the device and the
                               rows written into them directly, so that device
                               memory holds no result table; 0 = free device
                               memory less 2 GB [KNNSJ_DEVICE_TABLE_MB] */
  int32_t reserved[7];
} knnsj_options;

/* Statistics of one join (all optional to read). */
typedef struct {
  uint32_t struct_size;
  int32_t iterations;        /* search passes run */
  int32_t regrids;           /* grid rebuilds at a coarser cell width */
  int32_t eps_bucket;        /* histogram bucket that chose eps0 (GPU.cu:3510) */
  double eps0;               /* initial epsilon (DTYPE widened to double) */
  double eps_final;          /* largest radius searched */
  double avg_distance;       /* sampled mean pairwise distance (GPU.cu:3339) */
  double total_distance;     /* sum of squared kNN distances (GPU.cu:3690) */
  uint64_t candidates;       /* points scanned over all passes */
  uint64_t queries_run;      /* sum over passes of active queries */
  uint64_t nonempty_cells;   /* non-empty cells of the eps0 grid */
  double ms_total;           /* device time of the whole join */
  double ms_prep;            /* reorder + transpose + epsilon + grid */
  double ms_search;          /* all search passes */
  double ms_transfer;        /* host<->device copies (host-pointer calls; rows streamed into
                                pinned buffers during the join count where they outlast it) */
  uint32_t perm[64];         /* dimension order used (first min(d,64)) */
  uint64_t kernel_launches;  /* CUDA kernels launched by the join */
  double ms_search_kernels;  /* device time of the search kernel launches only */
  double search_alg_bytes;   /* algorithmic bytes of all search passes:
                                sum over passes of N*d*s + Q*d*s + accepted*(k+1)*(4+s) */
  double search_alg_flops;   /* 3*d per scanned candidate */
  double radius_model_error; /* KNNSJ_RADIUS_LEARNED: 0 ok; 1 the tensor-core radius model
                                timed out and the affected queries started at eps0 (rows stay
                                exact); 2 as 1, and a timed-out MMA was still unconfirmed when
                                its tensor memory was released */
  double tile_handovers;     /* queries the first pass's tile search handed to the per-query
                                search (ring far wider than its tile's, or exact ties) */
  double reserved[6];
} knnsj_stats;

/* One independent dataset of a batched call. */
typedef struct {
  const void* data;   /* row-major n x d, dtype of the call */
  uint64_t n;
  uint32_t d;
  uint32_t k;
  int32_t* out_ids;   /* n * (k+1) */
  void* out_dists;    /* n * (k+1) */
  knnsj_status status;/* written by the call */
} knnsj_set;

/* Library version string, e.g. "knnsj 1.0 (sm_103a)". */
const char* knnsj_version(void);

/* Human-readable status text. */
const char* knnsj_status_string(knnsj_status status);

/* DTYPE that KNNJoinPy was compiled with (params.h:5): KNNSJ_F32 or KNNSJ_F64. */
knnsj_dtype knnsj_build_dtype(void);

/* Replaces KNNJoinPy (main.cu:514-907) and the whole host pipeline behind it
 * -- ReorderByDimension (main.cu:2521), sampleNeighborsBruteForce
 * (GPU.cu:3088), generateNDGridDimensions (main.cu:2425),
 * populateNDGridIndexAndLookupArrayGPU (GPU.cu:3715) and the retry loop of
 * main.cu:705-823 around distanceTableNDGridBatcheskNN (GPU.cu:564).
 * Same symbol, argument meaning and output layout; DTYPE is the build's
 * (knnsj_build_dtype).  Like the reference it returns nothing: on a
 * dimension mismatch with a fixed-GPUNUMDIM build it prints the reference's
 * message and leaves the outputs untouched; on any other error it prints the
 * status and leaves row contents unspecified. */
#if defined(KNNSJ_KNNJOINPY_DOUBLE)
void KNNJoinPy(double* dataset, unsigned int NUMPOINTS, unsigned int kNN, unsigned int NDIM,
               int* outNearestNeighborTable, double* outNearestNeighborTableDistances);
#else
void KNNJoinPy(float* dataset, unsigned int NUMPOINTS, unsigned int kNN, unsigned int NDIM,
               int* outNearestNeighborTable, float* outNearestNeighborTableDistances);
#endif

/* Status-returning self-join on HOST buffers (same pipeline as KNNJoinPy,
 * dtype chosen per call).  data: row-major n x d; outputs as above.  When
 * both outputs are pinned and mapped (cudaHostAlloc, or cudaHostRegister
 * with cudaHostRegisterMapped), a kernel copies the device result table into
 * them through their mapped addresses after the join (KNNSJ_DIRECT_ROWS=1
 * instead has the search kernels write every row straight into them, with
 * no device result table; KNNSJ_DIRECT_ROWS=0 streams rows out of a device
 * table by the copy engines in KNNSJ_ROW_CHUNKS blocks of query ids while
 * the join runs).  Pageable outputs get a device result table copied out
 * after the join.  When the table would not fit in device memory (or
 * exceeds opts->device_table_mb), the outputs (pageable ones registered with
 * the device for the call) take their rows straight from the kernels: the
 * memory-bounded mode.  The call returns when every row is in place, also
 * on error (no kernel or copy is left writing into the outputs).  stats may
 * be NULL. */
knnsj_status knnsj_selfjoin(const void* data, knnsj_dtype dtype, uint64_t n, uint32_t d,
                            uint32_t k, const knnsj_options* opts, int32_t* out_ids,
                            void* out_dists, knnsj_stats* stats);

/* Same join on DEVICE-resident buffers of the current CUDA device: no host
 * copies.  All three pointers are device pointers. */
knnsj_status knnsj_selfjoin_device(const void* d_data, knnsj_dtype dtype, uint64_t n,
                                   uint32_t d, uint32_t k, const knnsj_options* opts,
                                   int32_t* d_out_ids, void* d_out_dists, knnsj_stats* stats);

/* No counterpart in the reference.  The device-buffer self-join for callers
 * that must not allocate GPU memory: runtimes whose own allocator owns the
 * device memory and forbids raw cudaMalloc/cudaFree, and hosts that fix every
 * device allocation up front (an allocation in the middle of their work could
 * fail or fragment their pool).  It calls no cudaMalloc, cudaFree, stream or
 * event creation and no allocating library routine; all scratch comes from
 * one static device array of KNNSJ_NOALLOC_SCRATCH_BYTES that every GPU
 * loading this library holds until the process exits.  Limits:
 * n <= KNNSJ_NOALLOC_MAX_POINTS, d <= 8, k+1 <= 128; larger problems return
 * KNNSJ_ERR_EXCEEDS_FIXED_SCRATCH, and so does any step of the join that
 * would need memory beyond the array.  The caller passes the input and output
 * device buffers, as for knnsj_selfjoin_device, and gets the same results.
 * The first call on a device looks up the array's device address
 * (cudaGetSymbolAddress); make that first call before any stream capture.
 * The call runs on the legacy default stream, reads a few small values back
 * to the host while it runs (stream synchronisations), and returns when the
 * join is done.  Every call reuses the same array, which keeps the previous
 * call's contents (the join clears what must start at zero); calls whose GPU
 * work overlapped would race on it, so the library takes its call lock and
 * finishes each call's GPU work before returning. */
#define KNNSJ_NOALLOC_SCRATCH_BYTES (24u << 20)
#define KNNSJ_NOALLOC_MAX_POINTS 65536u
knnsj_status knnsj_selfjoin_device_noalloc(const void* d_data, knnsj_dtype dtype, uint64_t n, uint32_t d,
                                           uint32_t k, const knnsj_options* opts, int32_t* d_out_ids,
                                           void* d_out_dists);

/* Many independent self-joins (host buffers), each with its own n, d, k and
 * results identical to a knnsj_selfjoin call on that set.  No reference
 * counterpart; replaces a loop of KNNJoinPy calls.  Returns the first
 * non-OK set status (each set's own status is written to sets[i].status). */
knnsj_status knnsj_selfjoin_batched(uint32_t n_sets, knnsj_set* sets, knnsj_dtype dtype,
                                    const knnsj_options* opts, knnsj_stats* stats);

/* Frees the device workspace cached by previous calls on the current device. */
void knnsj_release(void);

/* ---- learned starting radius (no reference counterpart) ----
 * A query's starting radius is eps0 * exp(MLP(features)), the MLP being
 * 24 -> 64 -> 64 -> 1 (ReLU, FP32); features and model layout are defined in
 * hybrid_k_nearest_neighbor_self_join_gb300/csrc/radius_model.cuh.  The
 * acceptance rule is unchanged, so results do not depend on the model. */
#define KNNSJ_RADIUS_FEATURES 24
#define KNNSJ_RADIUS_MODEL_FLOATS 5873

typedef struct {
  uint32_t struct_size;
  int32_t epochs;     /* passes over the samples (default 8) */
  uint32_t batch;     /* samples per Adam step (default 8192) */
  float lr;           /* Adam learning rate (default 1e-3) */
  float quantile;     /* pinball-loss quantile of log(r_K/eps0) (default 0.9) */
  uint64_t seed;      /* initialisation and shuffling seed */
} knnsj_train_options;

/* Copies the active model (KNNSJ_RADIUS_MODEL_FLOATS floats). */
knnsj_status knnsj_get_radius_model(float* out);
/* Replaces the active model; NULL restores the built-in one. */
knnsj_status knnsj_set_radius_model(const float* model);
/* Features of every point (row-major n x 24, by input row) on the eps0 grid
 * of a join of (data, k) with opts; *out_eps0 receives eps0. */
knnsj_status knnsj_radius_features(const void* data, knnsj_dtype dtype, uint64_t n, uint32_t d, uint32_t k,
                                   const knnsj_options* opts, float* out_features, double* out_eps0);
/* Model output for n feature rows (GPU). */
knnsj_status knnsj_radius_predict(const float* model, const float* features, uint64_t n, float* out);
/* Gradient of the mean pinball loss at `quantile` with respect to the
 * trainable parameters (the model from offset 48 on: 5825 floats) and the
 * loss itself, on n samples (GPU, deterministic). */
knnsj_status knnsj_radius_grad(const float* model, const float* features, const float* targets, uint64_t n,
                               float quantile, float* out_grad, double* out_loss);
/* Trains a model on (features, targets = log(r_K / eps0)) with Adam on the
 * GPU; loss_per_epoch (optional) receives the mean training loss per epoch. */
knnsj_status knnsj_radius_train(const float* features, const float* targets, uint64_t n,
                                const knnsj_train_options* opts, float* model_out, float* loss_per_epoch);

/* ---- host-side pieces of the reference pipeline (no GPU needed) ---- */

/* Dimension order of ReorderByDimension (main.cu:2521-2615): perm[j] is the
 * input dimension placed at slot j (descending sampled variance).
 * variances may be NULL. */
knnsj_status knnsj_reorder_dims(const void* data, knnsj_dtype dtype, uint64_t n, uint32_t d,
                                uint32_t* perm, void* variances);

/* Grid dimensions of generateNDGridDimensions (main.cu:2425-2488) over the
 * first di columns of row-major data: minArr/maxArr widened by eps and
 * nCells = ceil((max - min) / eps).  minArr, maxArr: di DTYPE values. */
knnsj_status knnsj_grid_dims(const void* data, knnsj_dtype dtype, uint64_t n, uint32_t d,
                             uint32_t di, double eps, void* minArr, void* maxArr,
                             uint32_t* nCells, uint64_t* totalCells);

/* CSV import with importNDDataset's tokenisation (import_dataset.cpp:50-106):
 * fields split on ',', each field read as whitespace-separated numbers until
 * the first that does not parse; every d consecutive values form a point and
 * a trailing partial point is dropped.  Two-call protocol: with out == NULL
 * only *n_points is written; then call again with out sized n_points * d. */
knnsj_status knnsj_read_csv(const char* path, knnsj_dtype dtype, uint32_t d, void* out,
                            uint64_t* n_points);

/* Outlier scores of a result table in DEVICE memory, on the GPU
 * (printOutlierScores, main.cu:952-1067): for each point q, mean[q] = the sum
 * of its K table distances (added in DTYPE in entry order) / (K - 1) in
 * double; dist_rank[q] = its position by decreasing sum; in_degree[q] = the
 * number of table entries naming q; degree_rank[q] = its position by
 * increasing in-degree.  Equal scores are ranked by point id (the reference
 * leaves them in std::sort's unspecified order; knnsj_write_outlier_scores
 * keeps that order for byte-identical files).  All pointers are device
 * pointers of the current device: ids/dists n*K, outputs n each. */
knnsj_status knnsj_outlier_scores_device(const int32_t* d_ids, const void* d_dists, knnsj_dtype dtype,
                                         uint64_t n, uint32_t K, double* d_mean, int32_t* d_dist_rank,
                                         uint64_t* d_in_degree, uint32_t* d_degree_rank);

/* Binary input (no reference counterpart: the reference reads CSV only,
 * import_dataset.cpp:50-106): a NumPy .npy file (format 1.0-3.0, C order,
 * little-endian float32 or float64, any shape; values converted to dtype) or,
 * without the .npy magic, raw little-endian values of dtype.  Every d
 * consecutive values form a point; a trailing partial point is dropped.
 * Same two-call protocol as knnsj_read_csv. */
knnsj_status knnsj_read_binary(const char* path, knnsj_dtype dtype, uint32_t d, void* out,
                               uint64_t* n_points);

/* KNN_out.txt and KNN_out_distances.txt in directory dir, in the format of
 * printNeighborTable (main.cu:911-949).  K = k+1 entries per row. */
knnsj_status knnsj_write_knn_out(const char* dir, uint64_t n, uint32_t K, const int32_t* ids,
                                 const void* dists, knnsj_dtype dtype);

/* KNN_outlier_scores.txt in directory dir, as printOutlierScores
 * (main.cu:952-1067): mean kNN distance, its rank, kNN in-degree, its rank. */
knnsj_status knnsj_write_outlier_scores(const char* dir, uint64_t n, uint32_t K,
                                        const int32_t* ids, const void* dists,
                                        knnsj_dtype dtype);

#ifdef __cplusplus
}
#endif

#endif /* KNNSJ_H */
