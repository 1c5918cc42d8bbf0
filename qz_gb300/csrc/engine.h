// Host-side engine for the block-sorting kernels: device scratch layout of one
// storage, and the forward / inverse drivers the C ABI (qzgpu.cu) wraps.
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

#include <atomic>
#include <condition_variable>
#include <cstring>
#include <functional>
#include <map>
#include <memory>
#include <thread>
#include <mutex>
#include <string>
#include <vector>

#include "common.cuh"

namespace qz {

// Segment classes of the per-round sort (by group length).
constexpr int kSmallMax = 16;    // longest group sorted by rank counting in a warp window
constexpr int kMedMax = 512;     // one warp sorts a group of up to kMedMax slots
constexpr int kOT = 4096;        // one CTA sorts a group of up to kOT slots; longer: onesweep tiles
constexpr int kInitTile = 4096;  // text positions per tile of the per-block passes
constexpr int kMaxRounds = 40;   // prefix doubling needs <= 31 rounds for n < 2^31

// Device counters (int32 slots of Storage::counters).  The ones a split
// writes are contiguous, so that one memset clears them before it.
enum Counter {
    CNT_ACTIVE = 0,  // suffixes still in non-singleton groups (two slots: 0 and 1,
                     // a split reads one and writes the other)
    CNT_ACTIVE_ALT = 1,
    CNT_LTILES = 2,  // tiles of the large-group radix sort
    CNT_TICKET = 3,  // tile tickets of a look-back radix pass
    CNT_SPLIT_FIRST = 4,
    CNT_MED = 4,     // descriptor counts of the listed classes
    CNT_LARGE = 5,
    CNT_MED_ELEMS = 6,  // slots covered by each listed class
    CNT_LARGE_ELEMS = 7,
    CNT_TILE = 8,
    CNT_TILE_ELEMS = 9,
    CNT_PAIR = 10,      // groups of 17..64 slots (rank-by-count class)
    CNT_PAIR_ELEMS = 11,
    CNT_SPLIT_TICKET = 12,  // warp-tile tickets of a one-pass split
    CNT_SPLIT_END = 13,
    CNT_SLOTS = 16,
};

struct FwdBuffers {
    int* SA;
    int* R;
    uint32_t* key;
    int* W[2];   // compact slots: suffix
    int* G[2];   // compact slots: group rank (SA position of the group's first slot)
    uint32_t* wsk[2];
    int* wsv[2];
    int2* list_rbc;    // groups of 17..64 slots (rank by count)
    int2* list_med;    // groups of 65..medium_max slots (warp radix)
    int2* list_tile;   // groups of 513..4096 slots
    int2* list_large;  // groups of more than 4096 slots
    uint8_t* straddle;  // per 32-slot window: a small group may cross its right boundary
    uint32_t* h4;      // large groups: digit counts of the four passes -> bases / pass-0 cursors
    unsigned long long* status64;  // look-back status per (tile, digit)
    uint32_t* gmask;   // large: per group, the passes whose digit is not constant
    uint32_t* ltc;     // large: tiles per group -> tile base
    uint32_t* llen;    // large: length per group -> workspace base
    uint32_t* ltbase;
    uint32_t* lwbase;
    uint32_t* tseg;    // large: group of each look-back tile
    int4* tdesc;       // large: per look-back tile, its group's descriptor (written by pass 0)
    int2* tdesc2;
    uint32_t* p_surv;  // split: per 256-slot warp tile
    int* p_sub;
    int* p_grp;
    unsigned long long* split_status;  // one-pass split: look-back words per warp tile
    uint32_t* c_surv;  // split: per scan chunk
    int* c_sub;
    int* c_grp;
};

struct InvBuffers {
    int* LF;
    int* next0;     // per ruler: ruler reached by walking LF (-1: row 0)
    int* len;       // per ruler: rows walked to reach it
    int* distF;     // per ruler: rows to row 0 once ranked
    int* hnext[2];  // per head (every 32nd ruler): next head and rows to it, ping-pong for jumping
    int* hdist[2];
    uint8_t* stage; // per ruler: the first-column symbols its walk passes (4 bytes per row of the stride)
    int* resume;    // per ruler: row where a walk longer than its staging slot stopped staging
    int2* rtiles;   // (block, first ruler) per walk tile
};

// Runtime tuning knobs of a lane (set through qzgpu_storage_set_param).
struct Tune {
    int big_ctas_per_sm = 3;   // persistent CTAs per SM of a look-back radix pass (1..4)
    int tile_ctas_per_sm = 3;  // CTAs of the one-CTA group sort
    int medium_max = kMedMax;  // longest group sorted by one warp (64..512)
    int ruler_log2 = 5;        // inverse: a ruler every 2^ruler_log2 rows (3..12)
    int big_tile = 4096;       // slots per look-back tile of the large-group sort (2048, 4096, 8192)
    int first_digit_max = 11;  // widest first radix digit of the large-group sort (8..11 bits)
    int round_pipeline = 0;    // forward rounds: 0 issued after the host reads their counts, 1 issued ahead
    int split_lookback = 0;    // split: 0 count + scan + apply passes, 1 one pass with decoupled look-back
    int rank_mode = 2;         // stable radix pass digit ranking: 0 warp match, 1 ballots, 2 match + ballots
    int early_counts = 0;      // stable radix pass: 1 digit counts published before the ranking
    int pass0_bulk = 1;        // radix pass 0: 1 double-buffered bulk copies of the next tile
    // failure-detection test: 1: in the first stable radix pass the second
    // tile of every group publishes nothing; 2: in every one-pass split the
    // second tile publishes nothing.  Look-back waits then give up after
    // 4096 polls, so the tiles after it report QZGPU_TIMEOUT (no GPU fault)
    int lookback_test = 0;
};

struct Storage {
    Tune tune;
    long long cap_bytes = 0;
    int cap_blocks = 0;
    int device = 0;
    int sms = 0;
    cudaStream_t stream = nullptr;  // internal stream for host-buffer calls

    // one device allocation, carved into the forward and inverse layouts
    char* dev = nullptr;
    size_t dev_bytes = 0;

    uint8_t* T = nullptr;  // staging copies for host-buffer calls
    uint8_t* U = nullptr;
    uint32_t* hist = nullptr;     // per-tile digit histograms (large sort / LF build)
    size_t hist_cap = 0;          // uint32 entries
    uint32_t* partial = nullptr;  // scan partials
    int* counters = nullptr;
    DevStatus* status = nullptr;

    // per-block tables
    int* blk_off = nullptr;     // nb + 1
    int* blk_K = nullptr;       // initial sort depth
    int* blk_sigma = nullptr;
    uint8_t* blk_code = nullptr;  // nb * 256 dense symbol codes
    uint32_t* blk_hist = nullptr; // nb * 256 byte counts
    int* blk_idx = nullptr;       // primary indexes out
    int* blk_status = nullptr;    // per-block result of an inverse (0 or a QZGPU_* code)
    int* blk_aux_rate = nullptr;
    int* blk_aux_off = nullptr;
    int* aux = nullptr;           // auxiliary indexes out
    int2* tiles = nullptr;        // (block, start) per kInitTile tile
    int* blk_tbase = nullptr;     // first tile of each block
    int* blk_hbase = nullptr;     // inverse: first ruler-list head of each block

    FwdBuffers f{};
    InvBuffers v{};

    // pinned host staging
    char* pin = nullptr;
    size_t pin_bytes = 0;
    char* pin_tab = nullptr;   // tables
    char* pin_tab_alt = nullptr;  // second table area (chained inverse sub-batches alternate)
    int* pin_rd = nullptr;     // small device->host readbacks
    size_t pin_tab_bytes = 0;
    // chained inverse sub-batches: the table area the next one fills, the
    // event after each area's last table copies, and work issued but not yet
    // checked
    int tab_slot = 0;
    cudaEvent_t tab_ev[2] = {nullptr, nullptr};
    bool inv_chained = false;

    std::mutex mu;
    qzgpu_stats stats{};
    int launches = 0;  // kernels launched by the current call

    // optional per-kernel timing (CUDA events around each launch)
    struct ProfRec {
        const char* name;
        cudaEvent_t a, b;
        long long bytes;
    };
    struct ProfAgg {
        int launches = 0;
        double ms = 0;
        long long bytes = 0;
    };
    bool profile = false;
    std::string profile_only;  // when set, only launches of this kernel are timed
    std::vector<cudaEvent_t> ev_pool;
    size_t ev_next = 0;
    std::vector<ProfRec> prof_pending;
    std::map<std::string, ProfAgg> prof;
    std::vector<long long> rounds_active;  // active suffixes per round of the last forward call
    long long sub_batch_bytes = 64ll << 20;  // forward: blocks grouped up to this size
    unsigned radix_epoch = 0;                // tags look-back status words of each pass
    cudaEvent_t round_ev[2] = {nullptr, nullptr};  // forward: counters of a split have landed
    // dry issue: launches are recorded (name, algorithmic bytes) instead of
    // made, to recompute a pipelined round's bytes from its exact counts
    bool dry = false;
    std::vector<std::pair<const char*, long long>> dry_list;
};

// Lane size of a multi-lane engine (block bytes one lane's sub-batch holds).
constexpr long long kLaneBytes = 64ll << 20;

// What callers hold as a qzgpu_storage: K lanes (scratch sets, each with its
// stream and worker thread) that take sub-batches of a call concurrently.
struct Engine {
    long long cap_bytes = 0;
    int cap_blocks = 0;
    long long lane_bytes = 0;
    int device = 0;
    std::vector<std::unique_ptr<Storage>> lanes;
    std::vector<std::thread> threads;
    std::mutex mu;  // one call at a time
    std::mutex jmu;
    std::condition_variable jcv, dcv;
    std::function<void(int)> job;
    int job_gen = 0, job_done = 0;
    bool stop = false;
    bool profile = false;
    std::string profile_only;  // when set, only launches of this kernel are timed
    // forward sub-batch size (<= lane_bytes): 16 MiB keeps a sub-batch's rank
    // array (64 MB) inside L2 next to the other lanes' random accesses; the
    // autotuner picked it on the chunk and on 256 uneven blocks
    long long fwd_sub_bytes = 16ll << 20;
    long long inv_sub_bytes = kLaneBytes;  // inverse sub-batch size (<= lane_bytes)
    qzgpu_stats stats{};
    std::vector<long long> rounds_active;
    std::map<std::string, Storage::ProfAgg> prof;
};

size_t engine_device_bytes(long long cap_bytes, int cap_blocks);
int engine_init(Engine* E, long long cap_bytes, int cap_blocks);
void engine_free(Engine* E);
// forward (true) or inverse of nb blocks: host buffers (hin/hout) or device
// buffers (d_in/d_out laid out back to back).  idx: per-block primary
// indexes (written by a forward call, read by an inverse call).
int engine_run(Engine* E, bool forward, int nb, const int* n, const unsigned char* const* hin,
               unsigned char* const* hout, const unsigned char* d_in, unsigned char* d_out, int* idx,
               cudaStream_t user_stream);

size_t storage_device_bytes(long long cap_bytes, int cap_blocks);
// Bytes of the inverse's ruler staging for a storage of this capacity.
size_t inverse_stage_bytes(long long cap_bytes, int cap_blocks);
int storage_init(Storage* S, long long cap_bytes, int cap_blocks);
void storage_free(Storage* S);

// Forward BWT of nb blocks laid out back to back in d_T (device).  n: host
// sizes.  idx (host, nb) receives primary indexes; aux_rate (host, may be
// null) selects per-block auxiliary index rates and aux_out (host, may be
// null) receives (n-1)/rate indexes per block, back to back.
int forward_run(Storage* S, int nb, const int* n, const uint8_t* d_T, uint8_t* d_U, int* idx,
                const int* aux_rate, int* aux_out, cudaStream_t st);

// Inverse BWT of nb blocks (d_U back to back, device) into d_T.  block_rc
// (host, nb entries, may be null) receives each block's own result when the
// call fails with QZGPU_DATA_CORRUPT: the blocks whose entry is 0 were
// inverted correctly, the others could not be inverted.
int inverse_run(Storage* S, int nb, const int* n, const int* idx, const uint8_t* d_U, uint8_t* d_T,
                cudaStream_t st, int* block_rc = nullptr);
// The same, issued without waiting for it (chained = true): the call returns
// once the work is queued on st.  Tables alternate between two pinned areas;
// the device status is neither cleared nor read, so a chain starts with
// inverse_chain_begin and ends with inverse_chain_end, which waits for the
// stream and returns the first failure of any link.
int inverse_run_chained(Storage* S, int nb, const int* n, const int* idx, const uint8_t* d_U, uint8_t* d_T,
                        cudaStream_t st);
void inverse_chain_begin(Storage* S, cudaStream_t st);
int inverse_chain_end(Storage* S, cudaStream_t st);

int map_cuda_error(cudaError_t e);
// The library's device (initialised on first use) and its SM count.
int device_info(int* device, int* sms);

// Host-buffer batch calls on a storage the caller holds (copies in, runs,
// copies out, synchronises the storage's stream).
int check_blocks(int nblocks, const int* n, long long* total);
// Host-buffer calls.  `before_copy_out`, when given, runs after the device
// work and before the device-to-host copies (the multi-lane engine waits there
// until the output pages have been touched).
int encode_host(Storage* S, int nb, const unsigned char* const* T, unsigned char* const* U, const int* n, int* idx,
                const int* aux_rate, int* aux_out, const std::function<void()>* before_copy_out = nullptr);
// block_rc (may be null): per-block results as for inverse_run; when it is
// given, a call that fails only for some blocks still copies every block out.
int decode_host(Storage* S, int nb, const unsigned char* const* U, unsigned char* const* T, const int* n,
                const int* idx, const std::function<void()>* before_copy_out = nullptr, int* block_rc = nullptr);
// A link of a chain of host-buffer inverse sub-batches on one storage (copies
// in, inverse, copies out, all queued on the storage's stream without a wait;
// see inverse_run_chained).  The caller's buffers must stay valid until
// inverse_chain_end.
int decode_host_chained(Storage* S, int nb, const unsigned char* const* U, unsigned char* const* T, const int* n,
                        const int* idx, const std::function<void()>* before_copy_out);

// Debug mode (environment QZGPU_DEBUG=1): every launch is followed by a
// stream synchronize and an error check, and failures are logged to stderr.
bool debug_on();
void debug_after(cudaStream_t st, const char* what);
void debug_log(const char* fmt, ...);
// Dump mode (environment QZGPU_DUMP=<dir>): writes device arrays of small
// batches to <dir>/<seq>_<name>.bin for offline inspection.
bool dump_on();
void dump_array(const char* name, const void* dptr, size_t bytes, cudaStream_t st);
cudaEvent_t prof_begin(Storage* S, cudaStream_t st, const char* name);
void prof_end(Storage* S, cudaStream_t st, const char* name, long long bytes, cudaEvent_t a);
void prof_flush(Storage* S);  // after the stream is idle: fold pending records in
// Raises kernel K's dynamic shared memory limit to `bytes` on the current
// device, once per device (the attribute belongs to the device; one bit per
// device number below 64, later devices set it at every launch).
template <auto K>
inline void smem_limit_once(int bytes, int device) {
    static std::atomic<unsigned long long> done{0};
    const unsigned long long bit = device >= 0 && device < 64 ? 1ull << device : 0ull;
    if (bit && (done.load(std::memory_order_acquire) & bit)) return;
    cudaFuncSetAttribute(K, cudaFuncAttributeMaxDynamicSharedMemorySize, bytes);
    done.fetch_or(bit, std::memory_order_acq_rel);
}

// Launch wrapper: counts the launch, times it when profiling, checks it in debug mode.
#define QZ_LAUNCH(S, st, name, bytes, ...)                     \
    do {                                                       \
        if ((S)->dry) {                                        \
            (S)->dry_list.emplace_back(name, (long long)(bytes)); \
            break;                                             \
        }                                                      \
        cudaEvent_t _qz_a = ::qz::prof_begin(S, st, name);     \
        __VA_ARGS__;                                           \
        ::qz::prof_end(S, st, name, (long long)(bytes), _qz_a); \
        QZ_DBG(st, name);                                      \
    } while (0)
#define QZ_DBG(st, what)                              \
    do {                                              \
        if (::qz::debug_on()) ::qz::debug_after(st, what); \
    } while (0)

}  // namespace qz
