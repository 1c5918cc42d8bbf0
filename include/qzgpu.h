/*
 * qzgpu — GB300 (sm_103a) block sorting for qz's BSC stage.
 *
 * C ABI only: plain pointers and sizes, no CUDA or torch types.  The entry
 * points below replace the block-sorting stage that qz reaches through
 * libbsc (crates/qz-lib/src/compression/bsc.rs:91-125):
 *
 *   - the forward BWT that bsc_compress runs on each block
 *     (called at bsc.rs:172-183 with blockSorter = LIBBSC_BLOCKSORTER_BWT);
 *   - the inverse BWT that bsc_decompress runs after the QLFC decoder
 *     (called at bsc.rs:421-433).
 *
 * libbsc's own BWT hooks (bsc_bwt_encode / bsc_bwt_decode in libbsc/bwt/bwt.h)
 * are not in the reference tree (third_party/ is git-ignored, .gitignore:31);
 * qzgpu_bwt_encode / qzgpu_bwt_decode keep their argument meaning: the block
 * is transformed in place in a caller-owned host buffer, the forward call
 * returns the primary index, and errors are libbsc's negative codes.
 *
 * Output convention (libsais, libbsc's CPU sorter): U[0] = T[n-1], followed by
 * the last column of the sorted suffix matrix with the sentinel row dropped;
 * primary index = 1 + rank of the whole block among its n non-empty suffixes.
 * Auxiliary index k (sampling rate r, a power of two) = 1 + rank of suffix k*r.
 *
 * Thread safety: every entry point may be called concurrently from many host
 * threads (qz calls the BSC wrapper from rayon workers, bsc.rs:285-288).
 */
#ifndef QZGPU_H
#define QZGPU_H

#ifdef __cplusplus
extern "C" {
#endif

/* Error codes: 0 and -1..-6 are libbsc's (bsc.rs:17-24); -7.. are GPU-side. */
#define QZGPU_NO_ERROR 0
#define QZGPU_BAD_PARAMETER (-1)
#define QZGPU_NOT_ENOUGH_MEMORY (-2)
#define QZGPU_NOT_COMPRESSIBLE (-3)
#define QZGPU_NOT_SUPPORTED (-4)
#define QZGPU_UNEXPECTED_EOB (-5)
#define QZGPU_DATA_CORRUPT (-6)
#define QZGPU_GPU_ERROR (-7)
#define QZGPU_GPU_NOT_SUPPORTED (-8)
#define QZGPU_GPU_NOT_ENOUGH_MEMORY (-9)
#define QZGPU_TIMEOUT (-10)
#define QZGPU_BLOCK_TOO_LARGE (-11)

/* libbsc feature bits (bsc.rs:32-36).  Accepted for signature compatibility;
 * the GPU path is always taken and never falls back to the CPU. */
#define QZGPU_FEATURE_FASTMODE 1
#define QZGPU_FEATURE_MULTITHREADING 2
#define QZGPU_FEATURE_LARGEPAGES 4
#define QZGPU_FEATURE_CUDA 8

/* Largest block one call accepts (libbsc's c_int limit, bsc.rs:165-167), and
 * the largest total of one device batch (keeps all positions in int32). */
#define QZGPU_MAX_BLOCK (1 << 30)
#define QZGPU_MAX_BATCH_BYTES (1LL << 30)

/* One-time initialisation; replaces bsc_init (bsc.rs:93, called once through
 * std::sync::Once at bsc.rs:128-141).  Selects the current CUDA device and
 * creates the shared scratch pool.  Idempotent; returns 0 or a negative code. */
int qzgpu_init(int features);

/* Human-readable name of an error code (never NULL). */
const char *qzgpu_error_string(int code);

/* ------------------------------------------------------------------------- */
/* libbsc BWT-stage drop-ins (host buffers, block transformed in place).       */
/* ------------------------------------------------------------------------- */

/* Forward BWT of T[0..n) in place; replaces libbsc's bsc_bwt_encode, which
 * bsc_compress runs for blockSorter = BWT (bsc.rs:172-183).  Returns the
 * primary index (>= 1; n for n <= 1) or a negative error.  When indexes is not
 * NULL, *num_indexes receives the auxiliary index count for rate
 * qzgpu_aux_rate(n) and indexes[0..*num_indexes) the indexes of suffixes
 * r, 2r, ... (indexes must hold 256 entries). */
int qzgpu_bwt_encode(unsigned char *T, int n, unsigned char *num_indexes, int *indexes, int features);

/* Inverse BWT of T[0..n) in place given the primary index; replaces libbsc's
 * bsc_bwt_decode, which bsc_decompress runs after QLFC decoding
 * (bsc.rs:421-433).  Auxiliary indexes are optional (num_indexes may be 0).
 * Returns 0, QZGPU_DATA_CORRUPT for an index or BWT that cannot be inverted,
 * or another negative code. */
int qzgpu_bwt_decode(unsigned char *T, int n, int index, unsigned char num_indexes, const int *indexes,
                     int features);

/* Auxiliary-index sampling rate used by qzgpu_bwt_encode for a block of n
 * bytes: the largest power of two <= max(n / 8, 1). */
int qzgpu_aux_rate(int n);

/* ------------------------------------------------------------------------- */
/* Device scratch storage (libcubwt-style: allocate once, reuse per call).     */
/* ------------------------------------------------------------------------- */

typedef struct qzgpu_storage qzgpu_storage;

/* Allocates device scratch for batches of up to max_total_bytes block bytes
 * and max_blocks blocks (about 60 bytes of HBM per block byte). */
int qzgpu_storage_create(qzgpu_storage **storage, long long max_total_bytes, int max_blocks);
int qzgpu_storage_destroy(qzgpu_storage *storage);

/* Device bytes one storage of this capacity allocates (for admission). */
long long qzgpu_storage_bytes(long long max_total_bytes, int max_blocks);

/* ------------------------------------------------------------------------- */
/* Batched forms: many blocks of uneven size in one set of launches.          */
/* ------------------------------------------------------------------------- */

/* Host buffers: forward BWT of blocks T[b][0..n[b]) into U[b] (U may equal T);
 * indexes[b] receives each primary index.  Replaces a rayon fan-out of
 * bsc_compress calls (compress_parallel_with, bsc.rs:259-301). */
int qzgpu_bwt_encode_batch(qzgpu_storage *storage, int nblocks, const unsigned char *const *T,
                           unsigned char *const *U, const int *n, int *indexes, int features);

/* Host buffers: inverse BWT of U[b] into T[b] (may alias).  Replaces the
 * parallel bsc_decompress fan-out of decompress_parallel (bsc.rs:324-371). */
int qzgpu_bwt_decode_batch(qzgpu_storage *storage, int nblocks, const unsigned char *const *U,
                           unsigned char *const *T, const int *n, const int *indexes, int features);

/* Device-resident form.  d_T / d_U hold the blocks back to back (block b at
 * offset n[0]+...+n[b-1]); n[] and indexes[] are host arrays.  Work is issued
 * on `stream` (a cudaStream_t, NULL for the legacy default stream); the call
 * returns once the results are final. */
int qzgpu_bwt_encode_device(qzgpu_storage *storage, int nblocks, const int *n, const unsigned char *d_T,
                            unsigned char *d_U, int *indexes, void *stream);
int qzgpu_bwt_decode_device(qzgpu_storage *storage, int nblocks, const int *n, const int *indexes,
                            const unsigned char *d_U, unsigned char *d_T, void *stream);

/* Counters from the last forward call on a storage. */
typedef struct qzgpu_stats {
    int rounds;               /* prefix-doubling rounds after the initial sort */
    int kernel_launches;      /* kernels this library launched for the call */
    long long active_total;   /* sum over rounds of suffixes still unsorted */
    long long alg_bytes;      /* algorithmic HBM bytes of the call */
} qzgpu_stats;
int qzgpu_storage_last_stats(const qzgpu_storage *storage, qzgpu_stats *out);

/* Suffixes sorted per round of the last forward call on a storage (entry 0:
 * the initial sort of every suffix; entry r: suffixes still in groups before
 * doubling round r).  Copies up to `max` entries; returns how many exist. */
int qzgpu_storage_round_counts(const qzgpu_storage *storage, long long *active, int max);

/* Runtime tuning of a storage (set by the autotuner, qz_gb300/autotune.py):
 *   "fwd_sub_bytes", "inv_sub_bytes"  block bytes per sub-batch taken by a lane
 *   "big_ctas_per_sm"                 persistent CTAs per SM of a radix pass (1..4)
 *   "tile_ctas_per_sm"                CTAs per SM of the one-CTA group sort (1..3)
 *   "medium_max"                      longest group sorted by one warp (64..512)
 *   "ruler_stride_log2"               inverse: a ruler every 2^v rows (3..12)
 *   "big_tile"                        slots per look-back tile of the large-group radix
 *                                     sort (2048, 4096, 8192)
 *   "radix_first_bits"                widest first (unstable) radix digit of that sort
 *                                     (8..11): keys of up to 16 + v bits sort in three
 *                                     passes, 8 keeps four passes above 24-bit keys
 *   "round_pipeline"                  forward doubling rounds: 0 each round issued after
 *                                     its counts are read back, 1 issued one round ahead
 *                                     with launch shapes from bounds
 *   "split_lookback"                  split after each group sort: 0 count, scan and
 *                                     apply passes (default), 1 one pass with decoupled
 *                                     look-back (less kernel time on one lane, slower
 *                                     when lanes overlap)
 *   "rank_mode"                       how a stable radix pass ranks a warp's digits:
 *                                     0 warp match, 1 eight ballots, 2 a match on the
 *                                     high four bits and four ballots (default)
 *   "early_counts"                    stable radix pass: 1 a tile publishes its digit
 *                                     counts for the look-back before it ranks, 0 after
 *                                     (default)
 *   "pass0_bulk"                      radix pass 0: 1 (default) each CTA loads its next
 *                                     tile by bulk copies while it sorts the current one,
 *                                     0 one tile at a time by 4-byte asynchronous copies
 *   "lookback_test"                  failure-detection test: forward calls fail with
 *                                     QZGPU_TIMEOUT through a bounded look-back wait that
 *                                     runs out, no GPU fault (1: in the radix sort, 2: in
 *                                     the one-pass split); 0: off (default)
 * get_param also answers "lanes".  Returns 0 / the value, or QZGPU_BAD_PARAMETER
 * for an unknown name or an out-of-range value.  No counterpart in libbsc. */
int qzgpu_storage_set_param(qzgpu_storage *storage, const char *name, long long value);
long long qzgpu_storage_get_param(const qzgpu_storage *storage, const char *name);

/* Per-kernel timing of later calls on a storage: when enabled, every launch
 * is bracketed by CUDA events on the stream it runs on.  Diagnostic only; no
 * counterpart in libbsc. */
typedef struct qzgpu_kernel_time {
    char name[32];
    int launches;
    double ms;              /* summed event-measured duration */
    long long alg_bytes;    /* summed algorithmic HBM bytes of those launches */
} qzgpu_kernel_time;
int qzgpu_storage_profile(qzgpu_storage *storage, int enable);
/* Restricts that timing to the launches of one kernel (by name; NULL or ""
 * times every kernel again), so that a long run is timed at little cost. */
int qzgpu_storage_profile_only(qzgpu_storage *storage, const char *name);
/* Copies up to `max` records (largest total time first); returns the number
 * of kernels recorded.  reset != 0 clears the records afterwards. */
int qzgpu_storage_profile_read(qzgpu_storage *storage, qzgpu_kernel_time *out, int max, int reset);

/* ------------------------------------------------------------------------- */
/* Serving: concurrent block requests, continuous batching on resident slots. */
/* ------------------------------------------------------------------------- */

/* Replaces per-block bsc_compress / bsc_decompress calls issued concurrently
 * by qz's rayon workers, chunk threads and decoder threads
 * (compress_impl.rs:364-387, decompress_impl.rs:666-689, bsc.rs:285-288):
 * requests from any host thread are batched onto device-resident slots. */
#define QZGPU_OP_FORWARD 0
#define QZGPU_OP_INVERSE 1

typedef struct qzgpu_server qzgpu_server;

/* Creates a server whose slots are device storages of slot_bytes block bytes
 * and slot_blocks blocks each (0 picks 64 MiB / 256).  It starts with one
 * slot and admits more on demand, at most max_slots (0: 4): while requests
 * wait and every slot is busy, one more slot is added when the slots' device
 * bytes (qzgpu_storage_bytes each) stay within hbm_budget_bytes (0: 80% of
 * the HBM free at creation) and the free HBM read at that moment covers the
 * slot plus a 256 MiB reserve; otherwise requests wait for a busy slot.  Each
 * slot has a worker thread and a stream; a free worker batches every waiting
 * request of one direction that fits its slot, in arrival order.  Returns
 * QZGPU_GPU_NOT_ENOUGH_MEMORY when not even one slot fits. */
int qzgpu_server_create(qzgpu_server **server, long long hbm_budget_bytes, int max_slots, long long slot_bytes,
                        int slot_blocks);
/* Number of slots the server holds now. */
int qzgpu_server_slots(const qzgpu_server *server);
/* Queues one block: op QZGPU_OP_FORWARD (in = block, out receives U) or
 * QZGPU_OP_INVERSE (in = U, index = primary index, out receives the block).
 * in/out stay owned by the caller until the request is waited for.  Returns a
 * ticket (>= 0) or a negative error. */
long long qzgpu_server_submit(qzgpu_server *server, int op, const unsigned char *in, unsigned char *out, int n,
                              int index);
/* Waits up to timeout_ms (< 0: forever) for a ticket.  Returns 1 when done
 * (status = the request's own result code, index_out = primary index of a
 * forward request, latency_ms = submit to completion, queue_ms = submit to
 * start of its batch; the ticket is then released), 0 on timeout (the ticket
 * can be waited for again), or a negative error: QZGPU_BAD_PARAMETER for an
 * unknown or released ticket, or one another thread is already waiting for.
 * Results are per request: an inverse request whose block cannot be inverted
 * gets QZGPU_DATA_CORRUPT while the other requests of its batch complete. */
int qzgpu_server_wait(qzgpu_server *server, long long ticket, int timeout_ms, int *status, int *index_out,
                      double *latency_ms, double *queue_ms);
/* Counters: completed requests, batches, largest batch, most slots busy at
 * once, requests waiting, slots, slot admissions refused for lack of free HBM
 * (or budget).  Returns the number of counters (7). */
int qzgpu_server_stats(const qzgpu_server *server, long long *out, int max);
/* Finishes every queued request, then frees the slots. */
int qzgpu_server_destroy(qzgpu_server *server);

/* ------------------------------------------------------------------------- */
/* Allocation-free inverse BWT.                                               */
/* ------------------------------------------------------------------------- */

/* Largest block qzgpu_bwt_decode_noalloc accepts (1 MiB). */
#define QZGPU_NOALLOC_MAX_BLOCK (1 << 20)

/* Inverse BWT of one block for callers that cannot allocate device memory
 * while they run (a host runtime that hands out all device memory up front
 * and forbids later cudaMalloc/cudaFree, or a thread that must not take the
 * allocator's locks).  No counterpart in the reference: libbsc's
 * bsc_bwt_decode allocates its own work arrays.
 *
 * d_U (input BWT) and d_T (output block) are device pointers of n bytes; they
 * may be the same buffer.  Work runs on `stream` (a cudaStream_t, NULL for the
 * legacy default stream); the call synchronizes that stream and returns when
 * the result is final.  It calls no cudaMalloc, cudaFree or other allocating
 * routine: its scratch is a fixed 6 MiB device array that every GPU loading
 * this library holds until the process exits.  The first call on a device
 * looks that array's address up (cudaGetSymbolAddress); make that first call
 * before any stream capture.  That address is not looked up again, so a
 * cudaDeviceReset in the process is not supported afterwards.  All calls in
 * the process share the array, so calls whose GPU work overlaps (other host
 * threads, other streams) race and must be serialised by the caller.  A CUDA
 * error already pending on the calling thread (from the caller's own work) is
 * left for the caller and the call returns QZGPU_GPU_ERROR without running.
 * Returns 0, QZGPU_BLOCK_TOO_LARGE for n > QZGPU_NOALLOC_MAX_BLOCK,
 * QZGPU_DATA_CORRUPT for an index or BWT that cannot be inverted, or another
 * negative code. */
int qzgpu_bwt_decode_noalloc(const unsigned char *d_U, unsigned char *d_T, int n, int index, void *stream);

/* ------------------------------------------------------------------------- */
/* Stream building on the device (the step before the block sorter).         */
/* ------------------------------------------------------------------------- */

/* Replaces records_to_streams (crates/qz-lib/src/compression/mod.rs:270-325)
 * on qz's default lossless BSC path (quality mode lossless, binning none:
 * 7 bits per quality, columnar.rs:16-36 and 104-134; no sequence hints, delta
 * or reverse-complement canonicalisation), together with the FASTQ reader that
 * feeds it (FastqReader::next, io/fastq.rs:135-200) and detect_const_lengths
 * (mod.rs:329-354): FASTQ text in, qz's three streams out.
 *
 *   header stream    [varint(len(id))][id]          (id: the '@' line)
 *   sequence stream  [varint(len) if lengths vary][bases]
 *   quality stream   [varint(len) if lengths vary][qualities, 7 bits each,
 *                    LSB first, min(max(q - 33, 0), 127), per read]
 *
 * Records follow the reader: four lines each, trailing '\r' trimmed, the third
 * line must start with '+', sequence and quality lengths must match, and an
 * input that ends inside a record is an error.  Returns 0,
 * QZGPU_DATA_CORRUPT for malformed input (info->error_record = the record the
 * reader fails on), or QZGPU_BAD_PARAMETER when an output capacity is below
 * the size in info (call with null outputs and zero capacities to size them).
 * Text up to 2 GiB - 1.  No counterpart in libbsc. */
typedef struct qzgpu_streams_info {
    long long records;
    long long header_bytes;
    long long seq_bytes;
    long long qual_bytes;
    int const_seq_len;   /* 0: lengths vary (length varints written) */
    int const_qual_len;
    long long error_record; /* -1 when the input is well formed */
} qzgpu_streams_info;
int qzgpu_fastq_streams(const unsigned char *fastq, long long n, unsigned char *header_out, long long header_cap,
                        unsigned char *seq_out, long long seq_cap, unsigned char *qual_out, long long qual_cap,
                        qzgpu_streams_info *info);

#ifdef __cplusplus
}
#endif

#endif /* QZGPU_H */
