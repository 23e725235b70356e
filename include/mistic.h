/*
 * mistic.h — C ABI of the GB300 ε-self-join library (libmistic.so).
 *
 * The reference (bwd29/self-join-MiSTIC) exposes its self-join only as a
 * command line, `build/main <file.bin> <dim> <numRP> <epsilon>`
 * (src/main.cu:20-50), over an internal C++ entry point
 *
 *   struct neighborTable* nodeLauncher5(double* data, unsigned dim,
 *       unsigned numPoints, unsigned numRP, unsigned* pointArray,
 *       double epsilon);                               (include/launcher.cuh:77-82)
 *
 * that builds the index (src/nodes.cu:5-356), runs the batched distance
 * kernel (src/kernel.cu:992-1046, launched at src/launcher.cu:3430), prints
 * "Total results Set Size: N" with N = ordered pairs including self pairs
 * (src/launcher.cu:3508-3515) and returns a per-point neighbour table
 * (include/utils.cuh:33-41).  The entry points below replace that function
 * and the CLI's data path: points, dimensionality d, reference-point count k
 * and ε go in; the pair count (both the reference's ordered-with-self number
 * and the unordered i<j count) and optionally the pair list come out.
 *
 * Conventions
 *  - Plain pointers and sizes only; no C++ or torch types cross this line.
 *  - Every function returns a mistic_status; nothing aborts or hangs.  A
 *    failing call leaves a message retrievable with mistic_last_error().
 *  - One handle owns one CUDA stream and its cached device buffers; calls on
 *    one handle must not overlap.  Different handles may be used from
 *    different host threads.
 *  - The caller owns the input; the library owns result buffers until
 *    mistic_result_free().
 *  - Row ids in pair lists are the caller's original row indices.
 *
 * The predicate is the reference's FP64 one (src/utils.cu:296-309 and
 * src/kernel.cu:833-865): s = Σ_k (x_k - y_k)^2 summed sequentially in column
 * order with each operation rounded, and a pair is in the result iff
 * s <= fl(ε*ε).  Every mode returns exactly that pair set: the reduced-
 * precision modes only pre-filter, and re-decide in FP64 every pair whose
 * fast distance lies inside a rigorous error band around ε².
 */
#ifndef MISTIC_H
#define MISTIC_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define MISTIC_ABI_VERSION 2

typedef enum mistic_status {
  MISTIC_OK = 0,
  MISTIC_ERR_INVALID_ARG = 1,   /* null pointer, d == 0, eps < 0 or not finite, ... */
  MISTIC_ERR_CUDA = 2,          /* a CUDA runtime call failed (see mistic_last_error) */
  MISTIC_ERR_OUT_OF_MEMORY = 3, /* device or pinned host allocation failed */
  MISTIC_ERR_TOO_LARGE = 4,     /* n >= 2^32 or d above the supported maximum */
  MISTIC_ERR_NOT_FINITE = 5,    /* an input coordinate is NaN or infinite */
  MISTIC_ERR_PAIR_OVERFLOW = 6, /* caller-sized pair buffer too small; counts are valid */
  MISTIC_ERR_TIMEOUT = 7,       /* a bounded device wait gave up; the context stays usable */
  MISTIC_ERR_NO_DEVICE = 8,     /* no CUDA device, or the device is not sm_103 */
  MISTIC_ERR_IO = 9,            /* file could not be read */
  MISTIC_ERR_INTERNAL = 10      /* device-side consistency check failed */
} mistic_status;

typedef enum mistic_dtype {
  MISTIC_F64 = 0, /* row-major n x d double (the reference's only format) */
  MISTIC_F32 = 1  /* row-major n x d float; widened exactly to FP64 for the predicate */
} mistic_dtype;

typedef enum mistic_mode {
  MISTIC_MODE_AUTO = 0, /* BF16 tensor-core mode for 8 <= d <= 126, else the FP32 filter */
  MISTIC_MODE_FP64 = 1, /* plain FP64 CUDA-core distances for every candidate */
  MISTIC_MODE_FP32 = 2, /* FP32 CUDA-core filter + FP64 re-decision of the band */
  MISTIC_MODE_BF16 = 3, /* large home bins as BF16 tensor-core Gram tiles (FP32
                           accumulation): split hi/lo operands, or, for long rows
                           (d + 2 > 128) when the bound leaves a narrow band, single
                           BF16 operands; small bins on the FP32 filter; FP64
                           re-decision of the band in both */
  MISTIC_MODE_TF32 = 4  /* large home bins as TF32 tensor-core Gram tiles (kind::tf32,
                           rows rounded to TF32 once, globally centred, FP32
                           accumulation), small bins on the FP32 filter; FP64
                           re-decision of the band.  Columns whose TF32 bound exceeds
                           eps^2 / 10 (small eps against the rows' norms) are decided
                           entirely in FP64, so BF16 is the faster choice there */
} mistic_mode;

typedef enum mistic_rp_mode {
  MISTIC_RP_PCA = 0,  /* k far points along the sample's top-k principal axes (default) */
  MISTIC_RP_BOX = 1,  /* k points uniform in the bounding box (seeded) */
  MISTIC_RP_USER = 2, /* caller-supplied k x d FP64 points in opts.rp_user */
  MISTIC_RP_SCORED = 3 /* the reference's per-layer selection (src/nodes.cu:168-222): layer by layer,
                          the candidate (far points along principal axes, sample points, box
                          points) leaving the fewest sample pairs within one eps-wide field on
                          every chosen layer */
} mistic_rp_mode;

typedef enum mistic_pairs_where {
  MISTIC_PAIRS_NONE = 0,   /* counts only; no pair list is materialised */
  MISTIC_PAIRS_HOST = 1,   /* result.pairs is a host array owned by the result (pinned memory
                              from a process-wide cache: release it with mistic_result_free) */
  MISTIC_PAIRS_DEVICE = 2  /* result.pairs is a device array owned by the result */
} mistic_pairs_where;

typedef struct mistic_opts {
  uint32_t struct_size;       /* = sizeof(mistic_opts); set by mistic_opts_init */
  mistic_mode mode;
  mistic_rp_mode rp_mode;
  const double* rp_user;      /* k x d host array when rp_mode == MISTIC_RP_USER */
  uint64_t seed;              /* seed for MISTIC_RP_BOX and PCA sampling */
  int32_t input_on_device;    /* 1: pts is a device pointer on the handle's device */
  mistic_pairs_where pairs;   /* where the pair list goes */
  int32_t sort_pairs;         /* 1: pair list sorted ascending by (i, j) */
  uint64_t pair_capacity;     /* 0: the library sizes the pair buffer itself */
  uint32_t* pair_buffer;      /* MISTIC_PAIRS_DEVICE only: caller-owned device buffer of
                                 pair_capacity pairs (2*pair_capacity uint32, 8-byte aligned),
                                 reused across calls like the reference's preallocated
                                 result arrays (src/launcher.cu:3340-3349); NULL: the
                                 library allocates and the result owns the list */
  int32_t check_finite;       /* 1 (default): reject NaN/inf inputs with MISTIC_ERR_NOT_FINITE */
  int32_t timing;             /* 1 (default): fill the per-phase times */
  mistic_pairs_where csr;     /* per-point neighbour table (CSR), the reference's neighborTable
                                 (include/utils.cuh:33-41, built in src/launcher.cu:4-50):
                                 NONE (default), HOST or DEVICE; see mistic_result.csr_* */
  uint32_t home_sample;       /* 0 or 1 (default): join every point.  S > 1: a sample at
                                 full density -- only the points of about 1 in S groups
                                 of 512 consecutive points of each bin's sorted order
                                 (picked by a hash of bin and group, the same in every
                                 mode) are joined as home points, each against all its
                                 candidates; counts, pair list and times cover that
                                 sample.  For comparing modes and tuning on a fixed
                                 subset of the work.  No counterpart in the reference. */
  int32_t autotune;           /* tensor-core join tuning (bin threshold, operand precision),
                                 timed on a sample of the work and cached per shape -- d,
                                 dtype, kernel, bin-size histogram class, eps against the
                                 rows' norms -- in memory and in the file MISTIC_TUNE_CACHE
                                 (default $HOME/.cache/mistic/tune.tsv): 0 (default) for
                                 joins of at least a million points, 1 always, -1 never.
                                 Replaces the reference's compile-time tunables
                                 (include/params.cuh:20-87). */
  uint64_t ring_capacity;     /* 0 (default): one pair list sized to the result.  R > 0: pairs
                                 stream through a device ring of R pairs (the reference keeps
                                 a fixed 2.5e9-pair buffer, src/launcher.cu:3340-3349, and
                                 nodeByPoint4 stops at 80 % of it, src/kernel.cu:912-989):
                                 when the ring fills, the join stops claiming work units, the
                                 ring is drained to the host (or to pair_sink), and the join
                                 resumes from its work cursor.  A unit that lost pairs to the
                                 full ring runs again in the next pass; its partial pairs are
                                 dropped (result.ring_units_redone).  Needs pairs = HOST or a
                                 pair_sink; no CSR table.  MISTIC_ERR_PAIR_OVERFLOW when one
                                 work unit alone has more pairs than the ring holds. */
  void (*pair_sink)(const uint32_t* pairs, uint64_t count, void* user);
                              /* ring mode: called on the calling thread with each drained
                                 batch of `count` pairs (i, j), i < j, in host memory valid
                                 for the call only; the result then holds no pair list */
  void* sink_user;
} mistic_opts;

typedef struct mistic_result {
  uint64_t n;                       /* points joined */
  uint32_t d, k_used;               /* k_used <= k: RPs that fit the 64-bit bin key */
  uint64_t pairs_ij;                /* unordered pairs i<j with s <= ε² */
  uint64_t pairs_ordered_incl_self; /* 2*pairs_ij + n: the reference's "Total results Set Size" */
  uint64_t candidates;              /* unordered candidate pairs the join evaluated */
  uint64_t band_pairs;              /* candidates re-decided in FP64 (0 in FP64 mode) */
  uint64_t ulp_ambiguous;           /* FP64-decided pairs with |s - ε²| <= 4 ulp(ε²) */
  uint64_t n_bins;                  /* non-empty bins of the reference-point index */
  uint64_t n_bin_pairs;             /* (home bin, neighbour bin) work items, home <= neighbour */
  uint64_t n_units;                 /* CUDA-core join work units after splitting */
  uint64_t n_units_tc;              /* tensor-core join work units (128-row home chunks) */
  uint64_t tc_tiles;                /* 128 x 128 tensor-core tiles evaluated */
  uint64_t tc_cells;                /* their occupied (home row, candidate) cells */
  uint32_t* pairs;                  /* 2*pairs_ij uint32 (i, j), i < j, or NULL */
  uint64_t pairs_len;               /* pairs stored (== pairs_ij unless capped) */
  int32_t pairs_on_device;
  mistic_mode mode_used;
  /* per-phase device times (CUDA events on the handle's stream), ms */
  double ms_total, ms_h2d, ms_prep, ms_keys, ms_sort, ms_bins, ms_enum, ms_join, ms_d2h;
  double ms_join_simt, ms_join_tc;  /* the two join kernels of the last join pass, ms */
  double ms_wall;                   /* host wall time of the whole call */
  uint32_t kernel_launches;         /* library kernels launched by this call */
  /* CSR neighbour table when opts.csr != NONE: the neighbours of row i are
   * csr_nbrs[csr_offsets[i] .. csr_offsets[i+1]), ascending, including i itself
   * as the reference's table does; csr_offsets[n] == pairs_ordered_incl_self. */
  uint64_t* csr_offsets;            /* n + 1 entries */
  uint32_t* csr_nbrs;               /* csr_offsets[n] entries */
  int32_t csr_on_device;
  int32_t tc_operands;              /* tensor-core operand precision used: 0 none, 1 split
                                       bf16 (hi/lo), 2 single bf16, 3 tf32 */
  uint32_t tc_min_bin;              /* smallest home bin joined on the tensor cores */
  int32_t tuned;                    /* 1: tc_min_bin / operands came from the autotuner
                                       (measured now, or cached for this shape) */
  uint32_t ring_passes;             /* ring mode: join passes (ring drains) */
  uint64_t ring_units_redone;       /* ring mode: units run again after the ring filled */
  int32_t tc_kernel;                /* tensor-core join used: 0 none, 1 short rows (per-unit
                                       centred operands converted per tile), 2 K-chunked (rows
                                       prepared once, globally centred) */
  void* _owner;                     /* internal: non-NULL when the result owns `pairs` */
} mistic_result;

typedef struct mistic_instance {   /* one self-join of a batch */
  const void* pts;
  uint64_t n;
  uint32_t d;
  mistic_dtype dtype;
  uint32_t k;
  double eps;
} mistic_instance;

typedef struct mistic_handle_s* mistic_handle;

/* Library/ABI version; lets a binding check it loaded a compatible build. */
int mistic_abi_version(void);

/* Fill opts with defaults (AUTO mode, PCA reference points, counts only). */
void mistic_opts_init(mistic_opts* opts);

/* Create a handle on `device`.  `stream` is a cudaStream_t to run on, or NULL
 * for a stream owned by the handle.  Replaces the reference's
 * cudaSetDevice(CUDA_DEVICE) + per-call allocations (src/main.cu:22,
 * src/launcher.cu:3259-3349). */
mistic_status mistic_create(mistic_handle* out, int device, void* stream);
mistic_status mistic_destroy(mistic_handle h);

/* The ε-self-join of n points (replaces nodeLauncher5, include/launcher.cuh:77-82,
 * and the join path of main, src/main.cu:20-182).  k is the number of
 * reference points of the bin index (the reference parses numRP at
 * src/main.cu:27 but always builds MAXRP = 6 layers, src/nodes.cu:62).
 * n == 0 and n == 1 are valid and yield zero pairs. */
mistic_status mistic_selfjoin(mistic_handle h, const void* pts, uint64_t n,
                              uint32_t d, mistic_dtype dtype, uint32_t k,
                              double eps, const mistic_opts* opts,
                              mistic_result* result);

/* m independent self-joins on one handle; results[i] receives instance i.
 * The reference has no batch entry point (one process per dataset,
 * script.sh:86-117); this replaces that loop. */
mistic_status mistic_batch_selfjoin(mistic_handle h, const mistic_instance* inst,
                                    uint32_t m, const mistic_opts* opts,
                                    mistic_result* results);

/* Read a raw little-endian row-major point file (the reference's input
 * format, src/main.cu:42-50: n = bytes / sizeof(elem) / d) into a malloc'd
 * host array released with mistic_free_host. */
mistic_status mistic_read_points(const char* path, uint32_t d, mistic_dtype dtype,
                                 void** out_pts, uint64_t* out_n);
void mistic_free_host(void* p);

/* GPU FP64 brute force over rows [row0, row1) against all n points: counts
 * [i - row0] = number of j != i whose reference predicate s(i, j) <= fl(ε*ε)
 * holds (src/utils.cu:296-309; the reference's GPU brute force is dumbBrute,
 * src/kernel.cu:1243-1261).  A subsample oracle at sizes where the CPU brute
 * force cannot run: for a sample of rows these counts must equal the
 * neighbour-table degrees minus the self edge.  `counts` is a host array of
 * row1 - row0 entries; `pts` is host memory unless input_on_device. */
mistic_status mistic_bruteforce_rows(mistic_handle h, const void* pts, uint64_t n, uint32_t d,
                                    mistic_dtype dtype, double eps, uint64_t row0, uint64_t row1,
                                    int input_on_device, uint32_t* counts);

/* Text -> binary converter with the behaviour of the reference's toBin tool
 * (toCSV.cpp:52-85): reads decimal numbers separated by commas and/or white
 * space from `text_path`, stopping at the first token that is not a number,
 * and writes them as raw little-endian FP64 to `bin_path` (the input format
 * of mistic_read_points and of the reference's main).  *out_count receives
 * the number of values written (may be NULL).  Host only; needs no GPU. */
mistic_status mistic_convert_text(const char* text_path, const char* bin_path, uint64_t* out_count);

/* Diagnostic with no counterpart in the reference: one 128 x 128 tensor-core
 * Gram tile D = A B^T (tcgen05.mma, FP32 accumulation in tensor memory,
 * issued exactly as the joins issue it), for measuring the accumulation error
 * that the joins' band bound allows for.  kind 0: a and b are 128 x K bf16
 * bit patterns (uint16, row-major, K a multiple of 16, K <= 256); kind 1:
 * 128 x K FP32 values read as tf32 (K a multiple of 8, K <= 128).  d receives
 * the 128 x 128 FP32 tile, row-major.  All pointers are host memory; runs on
 * the current device and returns when done. */
mistic_status mistic_tc_gram_probe(int kind, const void* a, const void* b, uint32_t K, float* d);

/* Release the buffers a result owns (pair list).  Safe on a zeroed result. */
void mistic_result_free(mistic_result* r);

const char* mistic_strerror(mistic_status s);
const char* mistic_last_error(mistic_handle h);

/* ---- No-allocation entry point.  This one has no counterpart in the
 * reference; it exists for callers that must not allocate device memory
 * while they run: a service whose device memory is reserved up front by its
 * own pool allocator (a fresh cudaMalloc can fail or fragment that pool), or
 * a latency-critical path where the implicit device-wide synchronisation of
 * cudaMalloc/cudaFree would stall other streams.
 *
 * The same exact ε-self-join (every pair i < j is a candidate: no reference-
 * point index, O(n^2) work, meant for modest n), with the points already on
 * the device (d_pts, row-major n x d) and the pair list written into the
 * caller's device buffer d_pairs (pair_capacity pairs of uint32 (i, j),
 * i < j, unsorted, 8-byte aligned).  *pairs_ij receives the pair count; the
 * call returns MISTIC_ERR_PAIR_OVERFLOW when it exceeds pair_capacity (the
 * count stays valid).  Runs on `stream` (a cudaStream_t, NULL = default
 * stream) on the current device and returns when the work is done.
 *
 * It calls no cudaMalloc/cudaFree and no allocating library routine: its only
 * scratch is one file-scope device array of MISTIC_NOALLOC_SCRATCH_BYTES
 * that every GPU which loads the library holds until the process exits.  The
 * scratch holds an FP32 copy of the points, so n * ceil4(d) * 4 bytes must fit
 * in it minus 256 bytes (e.g. n <= 419,427 at d = 18), and d must be at most
 * MISTIC_NOALLOC_MAX_D; larger inputs are rejected with MISTIC_ERR_TOO_LARGE.
 * The first call on a device looks up the array's device address
 * (cudaGetSymbolAddress) with that device current.  Under CUDA's default
 * lazy module loading the array is allocated
 * when the library's module first loads on the device, which is that first
 * call: make it before a pool allocator reserves the device's memory (a call
 * with n = 0 does only this set-up).  Inputs with a NaN or infinite
 * coordinate are rejected with MISTIC_ERR_NOT_FINITE.  All calls share the
 * array, so calls that overlap on the GPU (from several streams or host
 * threads) race; serialise them. */
#define MISTIC_NOALLOC_SCRATCH_BYTES (32u * 1024u * 1024u)
#define MISTIC_NOALLOC_MAX_D 128u
mistic_status mistic_selfjoin_noalloc(const void* d_pts, uint64_t n, uint32_t d, mistic_dtype dtype,
                                      double eps, uint32_t* d_pairs, uint64_t pair_capacity,
                                      uint64_t* pairs_ij, void* stream);

#ifdef __cplusplus
}
#endif

#endif /* MISTIC_H */
