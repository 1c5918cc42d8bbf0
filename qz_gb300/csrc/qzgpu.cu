// C ABI of the block-sorting library (declared in include/qzgpu.h): device
// scratch storages, a pool of them for the single-block libbsc-style calls,
// and host-buffer / device-buffer entry points.
#include <algorithm>
#include <cstdarg>
#include <cstdio>
#include <condition_variable>
#include <cstdlib>
#include <cstring>
#include <memory>
#include <mutex>
#include <vector>

#include "engine.h"
#include "radix.cuh"

namespace qz {

int map_cuda_error(cudaError_t e) {
    switch (e) {
        case cudaSuccess: return QZGPU_NO_ERROR;
        case cudaErrorMemoryAllocation: return QZGPU_GPU_NOT_ENOUGH_MEMORY;
        case cudaErrorNoDevice:
        case cudaErrorInsufficientDriver:
        case cudaErrorNoKernelImageForDevice: return QZGPU_GPU_NOT_SUPPORTED;
        default: return QZGPU_GPU_ERROR;
    }
}

bool debug_on() {
    static int on = -1;
    if (on < 0) {
        const char* e = getenv("QZGPU_DEBUG");
        on = (e && *e && *e != '0') ? 1 : 0;
    }
    return on == 1;
}

void debug_log(const char* fmt, ...) {
    va_list ap;
    va_start(ap, fmt);
    fprintf(stderr, "[qzgpu] ");
    vfprintf(stderr, fmt, ap);
    fprintf(stderr, "\n");
    va_end(ap);
}

void debug_after(cudaStream_t st, const char* what) {
    cudaError_t e = cudaGetLastError();
    if (e == cudaSuccess) e = cudaStreamSynchronize(st);
    if (e != cudaSuccess) debug_log("%s: %s", what, cudaGetErrorString(e));
}

cudaEvent_t prof_begin(Storage* S, cudaStream_t st, const char* name) {
    if (!S->profile) return nullptr;
    if (!S->profile_only.empty() && S->profile_only != name) return nullptr;
    if (S->ev_next + 2 > S->ev_pool.size()) {
        size_t grow = S->ev_pool.size() ? S->ev_pool.size() : 1024;
        for (size_t i = 0; i < grow; ++i) {
            cudaEvent_t e;
            if (cudaEventCreate(&e) != cudaSuccess) return nullptr;
            S->ev_pool.push_back(e);
        }
    }
    cudaEvent_t a = S->ev_pool[S->ev_next++];
    cudaEventRecord(a, st);
    return a;
}

// Launch log (environment QZGPU_LAUNCH_LOG=<file>): one line per launch,
// "name algorithmic_bytes", in the order the host issues them, so that a
// profiler's per-launch counters can be paired with the launches' own bytes.
static FILE* launch_log() {
    static FILE* f = [] {
        const char* p = getenv("QZGPU_LAUNCH_LOG");
        return (p && *p) ? fopen(p, "w") : nullptr;
    }();
    return f;
}

void prof_end(Storage* S, cudaStream_t st, const char* name, long long bytes, cudaEvent_t a) {
    ++S->launches;
    if (FILE* f = launch_log()) {
        static std::mutex mu;
        std::lock_guard<std::mutex> lk(mu);
        fprintf(f, "%s %lld\n", name, bytes);
        fflush(f);
    }
    if (!a) return;
    cudaEvent_t b = S->ev_pool[S->ev_next++];
    cudaEventRecord(b, st);
    S->prof_pending.push_back(Storage::ProfRec{name, a, b, bytes});
}

void prof_flush(Storage* S) {
    for (auto& r : S->prof_pending) {
        float ms = 0;
        if (cudaEventElapsedTime(&ms, r.a, r.b) != cudaSuccess) continue;
        auto& g = S->prof[r.name];
        g.launches += 1;
        g.ms += ms;
        g.bytes += r.bytes;
    }
    S->prof_pending.clear();
    S->ev_next = 0;
}

static const char* dump_dir() {
    static const char* d = getenv("QZGPU_DUMP");
    return (d && *d) ? d : nullptr;
}

bool dump_on() { return dump_dir() != nullptr; }

void dump_array(const char* name, const void* dptr, size_t bytes, cudaStream_t st) {
    static int seq = 0;
    if (!dump_dir()) return;
    std::vector<char> h(bytes);
    cudaStreamSynchronize(st);
    if (bytes && cudaMemcpy(h.data(), dptr, bytes, cudaMemcpyDeviceToHost) != cudaSuccess) {
        debug_log("dump %s: copy failed", name);
        return;
    }
    char path[1024];
    snprintf(path, sizeof(path), "%s/%04d_%s.bin", dump_dir(), seq++, name);
    FILE* f = fopen(path, "wb");
    if (!f) return;
    if (bytes) fwrite(h.data(), 1, bytes, f);
    fclose(f);
}

namespace {

constexpr size_t kAlign = 256;
constexpr int kMinStrideLog2 = 3;  // the inverse never uses rulers denser than every 8 rows

struct Carver {
    char* base;
    size_t off = 0;
    template <typename T>
    T* take(size_t count) {
        off = (off + kAlign - 1) / kAlign * kAlign;
        T* p = base ? reinterpret_cast<T*>(base + off) : nullptr;
        off += count * sizeof(T);
        return p;
    }
};

struct Caps {
    size_t N, nb, init_tiles, hist, med, tile, large, big_tiles, rulers, rtiles, aux;
};

Caps caps_for(long long cap_bytes, int cap_blocks) {
    Caps c;
    c.N = (size_t)cap_bytes;
    c.nb = (size_t)cap_blocks;
    c.init_tiles = c.N / kInitTile + c.nb + 1;
    // look-back tiles: sum over groups longer than kOT of ceil(len / kOT)
    size_t fwd_tiles = 2 * (c.N / kOT) + 2;
    c.hist = 256 * std::max(fwd_tiles, c.init_tiles);
    c.med = c.N / (kSmallMax + 1) + 1;
    c.tile = c.N / 65 + 2;  // medium_max may be tuned down to 64
    c.large = c.N / (kOT + 1) + 2;
    // look-back tiles of the large-group sort at its smallest tile (2048):
    // ceil(len / 2048) summed over groups longer than kOT
    c.big_tiles = c.N / 2048 + c.N / (kOT + 1) + 4;
    c.rulers = (c.N >> kMinStrideLog2) + c.nb + 1;
    c.rtiles = c.rulers / kThreads + c.nb + 1;
    c.aux = 64 * c.nb + 64;
    return c;
}

// Lays the device buffers out from `base` (null: only measure).
size_t layout(Storage* S, char* base, const Caps& c) {
    Carver cv{base};
    Storage tmp;
    Storage* s = S ? S : &tmp;
    s->T = cv.take<uint8_t>(c.N + 64);
    s->U = cv.take<uint8_t>(c.N + 64);
    s->hist = cv.take<uint32_t>(c.hist);
    s->hist_cap = c.hist;
    s->partial = cv.take<uint32_t>(1024);
    s->counters = cv.take<int>(64);
    s->status = cv.take<DevStatus>(1);
    s->blk_off = cv.take<int>(c.nb + 1);
    s->blk_K = cv.take<int>(c.nb + 1);
    s->blk_sigma = cv.take<int>(c.nb + 1);
    s->blk_code = cv.take<uint8_t>(256 * c.nb);
    s->blk_hist = cv.take<uint32_t>(256 * c.nb);
    s->blk_idx = cv.take<int>(c.nb + 1);
    s->blk_status = cv.take<int>(c.nb + 1);
    s->blk_aux_rate = cv.take<int>(c.nb + 1);
    s->blk_aux_off = cv.take<int>(c.nb + 1);
    s->blk_tbase = cv.take<int>(c.nb + 1);
    s->blk_hbase = cv.take<int>(c.nb + 1);
    s->aux = cv.take<int>(c.aux);
    s->tiles = cv.take<int2>(c.init_tiles);
    size_t shared_start = cv.off;
    // forward layout
    FwdBuffers& f = s->f;
    f.SA = cv.take<int>(c.N);
    f.R = cv.take<int>(c.N);
    f.key = cv.take<uint32_t>(c.N);
    for (int i = 0; i < 2; ++i) {
        f.W[i] = cv.take<int>(c.N);
        f.G[i] = cv.take<int>(c.N);
        f.wsk[i] = cv.take<uint32_t>(c.N);
        f.wsv[i] = cv.take<int>(c.N);
    }
    f.list_rbc = cv.take<int2>(c.med);
    f.list_med = cv.take<int2>(c.N / 65 + 2);
    f.straddle = cv.take<uint8_t>(c.N / 32 + 64);
    f.list_tile = cv.take<int2>(c.tile);
    f.list_large = cv.take<int2>(c.large);
    f.h4 = cv.take<uint32_t>(big_hist_words() * c.large);
    f.status64 = cv.take<unsigned long long>(256 * c.big_tiles);
    f.gmask = cv.take<uint32_t>(c.large + 1);
    f.ltc = cv.take<uint32_t>(c.large + 1);
    f.llen = cv.take<uint32_t>(c.large + 1);
    f.ltbase = cv.take<uint32_t>(c.large + 1);
    f.lwbase = cv.take<uint32_t>(c.large + 1);
    f.tseg = cv.take<uint32_t>(c.big_tiles);
    f.tdesc = cv.take<int4>(c.big_tiles);
    f.tdesc2 = cv.take<int2>(c.big_tiles);
    size_t wt = c.N / 256 + 2;
    f.p_surv = cv.take<uint32_t>(wt);
    f.p_sub = cv.take<int>(wt);
    f.p_grp = cv.take<int>(wt);
    f.split_status = cv.take<unsigned long long>(4 * wt);
    f.c_surv = cv.take<uint32_t>(1024);
    f.c_sub = cv.take<int>(1024);
    f.c_grp = cv.take<int>(1024);
    size_t fwd_end = cv.off;
    // inverse layout, aliasing the forward buffers
    cv.off = shared_start;
    InvBuffers& v = s->v;
    v.LF = cv.take<int>(c.N + c.nb + 1);
    v.next0 = cv.take<int>(c.rulers);
    v.len = cv.take<int>(c.rulers);
    v.distF = cv.take<int>(c.rulers);
    const size_t heads = c.rulers / 32 + c.nb + 1;
    for (int i = 0; i < 2; ++i) {
        v.hnext[i] = cv.take<int>(heads);
        v.hdist[i] = cv.take<int>(heads);
    }
    v.stage = cv.take<uint8_t>(inverse_stage_bytes((long long)c.N, (int)c.nb));
    v.resume = cv.take<int>(c.rulers);
    v.rtiles = cv.take<int2>(c.rtiles);
    return std::max(fwd_end, cv.off) + kAlign;
}

size_t pinned_table_bytes(const Caps& c) {
    return sizeof(int) * 8 * (c.nb + 1) + sizeof(int2) * (c.init_tiles + c.rtiles + 3 * c.nb + 8) +
           sizeof(int) * 64 + 4096;
}

// ---------------------------------------------------------------- global state

struct Global {
    std::mutex mu;
    bool inited = false;
    int device = 0;
    int sms = 0;
    // pool of storages for the single-block drop-in calls
    std::condition_variable cv;
    std::vector<std::unique_ptr<Storage>> pool;
    std::vector<Storage*> idle;
    int pool_max = 4;
    long long pool_cap = 32ll << 20;  // covers qz's 25 MiB blocks
};

Global& G() {
    static Global g;
    return g;
}

int ensure_init() {
    Global& g = G();
    std::lock_guard<std::mutex> lk(g.mu);
    if (g.inited) return QZGPU_NO_ERROR;
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) return map_cuda_error(e);
    int sms = 0;
    e = cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    if (e != cudaSuccess) return map_cuda_error(e);
    g.device = dev;
    g.sms = sms;
    g.inited = true;
    const char* env = getenv("QZGPU_POOL_STORAGES");
    if (env && atoi(env) > 0) g.pool_max = atoi(env);
    return QZGPU_NO_ERROR;
}

Storage* pool_acquire(long long need) {
    Global& g = G();
    std::unique_lock<std::mutex> lk(g.mu);
    for (;;) {
        for (size_t i = 0; i < g.idle.size(); ++i) {
            if (g.idle[i]->cap_bytes >= need) {
                Storage* s = g.idle[i];
                g.idle.erase(g.idle.begin() + (long)i);
                return s;
            }
        }
        if ((int)g.pool.size() < g.pool_max) {
            auto s = std::make_unique<Storage>();
            lk.unlock();
            int rc = storage_init(s.get(), std::max(need, g.pool_cap), 1);
            lk.lock();
            if (rc != QZGPU_NO_ERROR) return nullptr;
            g.pool.push_back(std::move(s));
            return g.pool.back().get();
        }
        g.cv.wait(lk);
    }
}

void pool_release(Storage* s) {
    Global& g = G();
    {
        std::lock_guard<std::mutex> lk(g.mu);
        g.idle.push_back(s);
    }
    g.cv.notify_one();
}

}  // namespace

size_t storage_device_bytes(long long cap_bytes, int cap_blocks) {
    return layout(nullptr, nullptr, caps_for(cap_bytes, cap_blocks));
}

int storage_init(Storage* S, long long cap_bytes, int cap_blocks) {
    int rc = ensure_init();
    if (rc) return rc;
    if (cap_bytes < 1 || cap_blocks < 1 || cap_bytes > QZGPU_MAX_BATCH_BYTES) return QZGPU_BAD_PARAMETER;
    Global& g = G();
    cudaError_t e = cudaSetDevice(g.device);
    if (e != cudaSuccess) return map_cuda_error(e);
    Caps c = caps_for(cap_bytes, cap_blocks);
    S->cap_bytes = cap_bytes;
    S->cap_blocks = cap_blocks;
    const char* sb = getenv("QZGPU_SUB_BATCH_MB");
    if (sb && atof(sb) > 0) S->sub_batch_bytes = (long long)(atof(sb) * (1 << 20));
    S->device = g.device;
    S->sms = g.sms;
    size_t bytes = layout(nullptr, nullptr, c);
    e = cudaMalloc(&S->dev, bytes);
    if (e != cudaSuccess) {
        S->dev = nullptr;
        return map_cuda_error(e);
    }
    S->dev_bytes = bytes;
    layout(S, S->dev, c);
    S->pin_tab_bytes = (pinned_table_bytes(c) + 255) / 256 * 256;
    size_t rd = sizeof(int) * (c.nb + 256);
    S->pin_bytes = 2 * S->pin_tab_bytes + rd + 64;
    e = cudaMallocHost(&S->pin, S->pin_bytes);
    if (e != cudaSuccess) {
        cudaFree(S->dev);
        S->dev = nullptr;
        S->pin = nullptr;
        return QZGPU_NOT_ENOUGH_MEMORY;
    }
    S->pin_tab = S->pin;
    S->pin_tab_alt = S->pin + S->pin_tab_bytes;
    S->pin_rd = reinterpret_cast<int*>(S->pin_tab_alt + S->pin_tab_bytes);
    e = cudaStreamCreateWithFlags(&S->stream, cudaStreamNonBlocking);
    for (int i = 0; i < 2 && e == cudaSuccess; ++i) e = cudaEventCreateWithFlags(&S->round_ev[i], cudaEventDisableTiming);
    for (int i = 0; i < 2 && e == cudaSuccess; ++i) e = cudaEventCreateWithFlags(&S->tab_ev[i], cudaEventDisableTiming);
    if (e != cudaSuccess) {
        storage_free(S);
        return map_cuda_error(e);
    }
    return QZGPU_NO_ERROR;
}

void storage_free(Storage* S) {
    for (auto e : S->ev_pool) cudaEventDestroy(e);
    S->ev_pool.clear();
    for (auto& e : S->round_ev) {
        if (e) cudaEventDestroy(e);
        e = nullptr;
    }
    for (auto& e : S->tab_ev) {
        if (e) cudaEventDestroy(e);
        e = nullptr;
    }
    if (S->stream) cudaStreamDestroy(S->stream);
    if (S->dev) cudaFree(S->dev);
    if (S->pin) cudaFreeHost(S->pin);
    S->stream = nullptr;
    S->dev = nullptr;
    S->pin = nullptr;
}

}  // namespace qz

using namespace qz;

struct qzgpu_storage : public qz::Engine {};

namespace qz {

int check_blocks(int nblocks, const int* n, long long* total) {
    if (nblocks < 0 || (nblocks > 0 && !n)) return QZGPU_BAD_PARAMETER;
    long long t = 0;
    for (int b = 0; b < nblocks; ++b) {
        if (n[b] < 0 || n[b] > QZGPU_MAX_BLOCK) return QZGPU_BAD_PARAMETER;
        t += n[b];
    }
    *total = t;
    return QZGPU_NO_ERROR;
}

// Host-buffer forward batch on storage S (caller holds S->mu).
int encode_host(Storage* S, int nb, const unsigned char* const* T, unsigned char* const* U, const int* n,
                int* idx, const int* aux_rate, int* aux_out, const std::function<void()>* before_copy_out) {
    cudaError_t e = cudaSetDevice(S->device);
    if (e != cudaSuccess) return map_cuda_error(e);
    long long off = 0;
    for (int b = 0; b < nb; ++b) {
        if (n[b] > 0) {
            e = cudaMemcpyAsync(S->T + off, T[b], (size_t)n[b], cudaMemcpyHostToDevice, S->stream);
            if (e != cudaSuccess) return map_cuda_error(e);
        }
        off += n[b];
    }
    int rc = forward_run(S, nb, n, S->T, S->U, idx, aux_rate, aux_out, S->stream);
    if (rc) return rc;
    if (before_copy_out) (*before_copy_out)();
    off = 0;
    for (int b = 0; b < nb; ++b) {
        if (n[b] > 0) {
            e = cudaMemcpyAsync(U[b], S->U + off, (size_t)n[b], cudaMemcpyDeviceToHost, S->stream);
            if (e != cudaSuccess) return map_cuda_error(e);
        }
        off += n[b];
    }
    e = cudaStreamSynchronize(S->stream);
    return map_cuda_error(e);
}

int decode_host(Storage* S, int nb, const unsigned char* const* U, unsigned char* const* T, const int* n,
                const int* idx, const std::function<void()>* before_copy_out, int* block_rc) {
    cudaError_t e = cudaSetDevice(S->device);
    if (e != cudaSuccess) return map_cuda_error(e);
    long long off = 0;
    for (int b = 0; b < nb; ++b) {
        if (n[b] > 0) {
            e = cudaMemcpyAsync(S->U + off, U[b], (size_t)n[b], cudaMemcpyHostToDevice, S->stream);
            if (e != cudaSuccess) return map_cuda_error(e);
        }
        off += n[b];
    }
    const int rc = inverse_run(S, nb, n, idx, S->U, S->T, S->stream, block_rc);
    // a failure of some blocks only (block_rc says which): the others are final
    if (rc && !(rc == QZGPU_DATA_CORRUPT && block_rc)) return rc;
    if (before_copy_out) (*before_copy_out)();
    off = 0;
    for (int b = 0; b < nb; ++b) {
        if (n[b] > 0 && !(block_rc && block_rc[b])) {
            e = cudaMemcpyAsync(T[b], S->T + off, (size_t)n[b], cudaMemcpyDeviceToHost, S->stream);
            if (e != cudaSuccess) return map_cuda_error(e);
        }
        off += n[b];
    }
    e = cudaStreamSynchronize(S->stream);
    return e != cudaSuccess ? map_cuda_error(e) : rc;
}

int decode_host_chained(Storage* S, int nb, const unsigned char* const* U, unsigned char* const* T, const int* n,
                        const int* idx, const std::function<void()>* before_copy_out) {
    cudaError_t e = cudaSetDevice(S->device);
    if (e != cudaSuccess) return map_cuda_error(e);
    long long off = 0;
    for (int b = 0; b < nb; ++b) {
        if (n[b] > 0) {
            e = cudaMemcpyAsync(S->U + off, U[b], (size_t)n[b], cudaMemcpyHostToDevice, S->stream);
            if (e != cudaSuccess) return map_cuda_error(e);
        }
        off += n[b];
    }
    const int rc = inverse_run_chained(S, nb, n, idx, S->U, S->T, S->stream);
    if (rc) return rc;
    if (before_copy_out) (*before_copy_out)();
    off = 0;
    for (int b = 0; b < nb; ++b) {
        if (n[b] > 0) {
            e = cudaMemcpyAsync(T[b], S->T + off, (size_t)n[b], cudaMemcpyDeviceToHost, S->stream);
            if (e != cudaSuccess) return map_cuda_error(e);
        }
        off += n[b];
    }
    return QZGPU_NO_ERROR;
}

int device_info(int* device, int* sms) {
    int rc = ensure_init();
    if (rc) return rc;
    *device = G().device;
    *sms = G().sms;
    return QZGPU_NO_ERROR;
}

}  // namespace qz

namespace {

// Runs fn on a pooled storage that fits `need` bytes (or a temporary one).
template <typename Fn>
int with_pooled(long long need, Fn fn) {
    int rc = ensure_init();
    if (rc) return rc;
    if (need > G().pool_cap) {
        Storage tmp;
        rc = storage_init(&tmp, need, 1);
        if (rc) return rc;
        rc = fn(&tmp);
        storage_free(&tmp);
        return rc;
    }
    Storage* s = pool_acquire(need);
    if (!s) return QZGPU_GPU_NOT_ENOUGH_MEMORY;
    {
        std::lock_guard<std::mutex> lk(s->mu);
        rc = fn(s);
    }
    pool_release(s);
    return rc;
}

}  // namespace

extern "C" {

int qzgpu_init(int features) {
    (void)features;
    return ensure_init();
}

const char* qzgpu_error_string(int code) {
    switch (code) {
        case QZGPU_NO_ERROR: return "no error";
        case QZGPU_BAD_PARAMETER: return "bad parameter";
        case QZGPU_NOT_ENOUGH_MEMORY: return "not enough host memory";
        case QZGPU_NOT_COMPRESSIBLE: return "not compressible";
        case QZGPU_NOT_SUPPORTED: return "not supported";
        case QZGPU_UNEXPECTED_EOB: return "unexpected end of block";
        case QZGPU_DATA_CORRUPT: return "data corrupt";
        case QZGPU_GPU_ERROR: return "GPU error";
        case QZGPU_GPU_NOT_SUPPORTED: return "no usable GPU";
        case QZGPU_GPU_NOT_ENOUGH_MEMORY: return "not enough GPU memory";
        case QZGPU_TIMEOUT: return "timed out";
        case QZGPU_BLOCK_TOO_LARGE: return "block larger than this entry point accepts";
        default: return "unknown error";
    }
}

int qzgpu_aux_rate(int n) {
    int x = n / 8;
    if (x < 1) return 1;
    int r = 1;
    while ((r << 1) <= x) r <<= 1;
    return r;
}

int qzgpu_bwt_encode(unsigned char* T, int n, unsigned char* num_indexes, int* indexes, int features) {
    (void)features;
    if (n < 0 || (n > 0 && !T)) return QZGPU_BAD_PARAMETER;
    if (num_indexes) *num_indexes = 0;
    if (n <= 1) return n;
    int rate = qzgpu_aux_rate(n);
    int naux = (n - 1) / rate;
    bool want_aux = indexes && num_indexes && naux <= 255;
    int idx = 0;
    int rc = with_pooled(n, [&](Storage* s) {
        const unsigned char* in[1] = {T};
        unsigned char* out[1] = {T};
        return encode_host(s, 1, in, out, &n, &idx, want_aux ? &rate : nullptr, want_aux ? indexes : nullptr);
    });
    if (rc) return rc;
    if (want_aux) *num_indexes = (unsigned char)naux;
    return idx;
}

int qzgpu_bwt_decode(unsigned char* T, int n, int index, unsigned char num_indexes, const int* indexes,
                     int features) {
    (void)features;
    (void)num_indexes;
    (void)indexes;
    if (n < 0 || (n > 0 && !T)) return QZGPU_BAD_PARAMETER;
    if (n == 0) return QZGPU_NO_ERROR;
    if (index < 1 || index > n) return QZGPU_DATA_CORRUPT;
    if (n == 1) return QZGPU_NO_ERROR;
    return with_pooled(n, [&](Storage* s) {
        const unsigned char* in[1] = {T};
        unsigned char* out[1] = {T};
        return decode_host(s, 1, in, out, &n, &index);
    });
}

long long qzgpu_storage_bytes(long long max_total_bytes, int max_blocks) {
    if (max_total_bytes < 1 || max_blocks < 1) return 0;
    return (long long)engine_device_bytes(max_total_bytes, max_blocks);
}

int qzgpu_storage_create(qzgpu_storage** storage, long long max_total_bytes, int max_blocks) {
    if (!storage) return QZGPU_BAD_PARAMETER;
    *storage = nullptr;
    if (max_total_bytes < 1 || max_blocks < 1 || max_total_bytes > QZGPU_MAX_BATCH_BYTES) return QZGPU_BAD_PARAMETER;
    auto* s = new (std::nothrow) qzgpu_storage();
    if (!s) return QZGPU_NOT_ENOUGH_MEMORY;
    int rc = engine_init(s, max_total_bytes, max_blocks);
    if (rc) {
        delete s;
        return rc;
    }
    *storage = s;
    return QZGPU_NO_ERROR;
}

int qzgpu_storage_destroy(qzgpu_storage* storage) {
    if (!storage) return QZGPU_BAD_PARAMETER;
    {
        std::lock_guard<std::mutex> lk(storage->mu);
        engine_free(storage);
    }
    delete storage;
    return QZGPU_NO_ERROR;
}

namespace {

int engine_call(qzgpu_storage* storage, bool forward, int nblocks, const int* n, const unsigned char* const* hin,
                unsigned char* const* hout, const unsigned char* d_in, unsigned char* d_out, int* idx, void* stream) {
    long long total;
    int rc = check_blocks(nblocks, n, &total);
    if (rc) return rc;
    if (!storage) return QZGPU_BAD_PARAMETER;
    bool host = hin != nullptr;
    if (nblocks > 0 && !idx) return QZGPU_BAD_PARAMETER;
    if (host && nblocks > 0 && !hout) return QZGPU_BAD_PARAMETER;
    if (!host && total > 0 && (!d_in || !d_out || d_in == d_out)) return QZGPU_BAD_PARAMETER;
    if (!forward)
        for (int b = 0; b < nblocks; ++b)
            if (n[b] > 0 && (idx[b] < 1 || idx[b] > n[b])) return QZGPU_DATA_CORRUPT;
    std::lock_guard<std::mutex> lk(storage->mu);
    if (total > storage->cap_bytes || nblocks > storage->cap_blocks) return QZGPU_BAD_PARAMETER;
    cudaError_t e = cudaSetDevice(storage->device);
    if (e != cudaSuccess) return map_cuda_error(e);
    return engine_run(storage, forward, nblocks, n, hin, hout, d_in, d_out, idx,
                      reinterpret_cast<cudaStream_t>(stream));
}

}  // namespace

int qzgpu_bwt_encode_batch(qzgpu_storage* storage, int nblocks, const unsigned char* const* T,
                           unsigned char* const* U, const int* n, int* indexes, int features) {
    (void)features;
    if (nblocks > 0 && (!T || !U)) return QZGPU_BAD_PARAMETER;
    return engine_call(storage, true, nblocks, n, nblocks > 0 ? T : (const unsigned char* const*)&T, U, nullptr,
                       nullptr, indexes, nullptr);
}

int qzgpu_bwt_decode_batch(qzgpu_storage* storage, int nblocks, const unsigned char* const* U,
                           unsigned char* const* T, const int* n, const int* indexes, int features) {
    (void)features;
    if (nblocks > 0 && (!T || !U)) return QZGPU_BAD_PARAMETER;
    return engine_call(storage, false, nblocks, n, nblocks > 0 ? U : (const unsigned char* const*)&U, T, nullptr,
                       nullptr, const_cast<int*>(indexes), nullptr);
}

int qzgpu_bwt_encode_device(qzgpu_storage* storage, int nblocks, const int* n, const unsigned char* d_T,
                            unsigned char* d_U, int* indexes, void* stream) {
    return engine_call(storage, true, nblocks, n, nullptr, nullptr, d_T, d_U, indexes, stream);
}

int qzgpu_bwt_decode_device(qzgpu_storage* storage, int nblocks, const int* n, const int* indexes,
                            const unsigned char* d_U, unsigned char* d_T, void* stream) {
    return engine_call(storage, false, nblocks, n, nullptr, nullptr, d_U, d_T, const_cast<int*>(indexes), stream);
}

int qzgpu_storage_set_param(qzgpu_storage* storage, const char* name, long long value) {
    if (!storage || !name) return QZGPU_BAD_PARAMETER;
    std::lock_guard<std::mutex> lk(storage->mu);
    std::string k(name);
    auto each = [&](auto fn) {
        for (auto& l : storage->lanes) fn(l->tune);
    };
    if (k == "fwd_sub_bytes" || k == "inv_sub_bytes") {
        if (value < (1 << 20)) return QZGPU_BAD_PARAMETER;
        (k[0] == 'f' ? storage->fwd_sub_bytes : storage->inv_sub_bytes) = value;
    } else if (k == "big_ctas_per_sm") {
        // a tile waits only on tiles of earlier tickets, which resident CTAs
        // hold, so CTAs beyond residency only queue
        if (value < 1 || value > 4) return QZGPU_BAD_PARAMETER;
        each([&](Tune& t) { t.big_ctas_per_sm = (int)value; });
    } else if (k == "tile_ctas_per_sm") {
        if (value < 1 || value > 3) return QZGPU_BAD_PARAMETER;
        each([&](Tune& t) { t.tile_ctas_per_sm = (int)value; });
    } else if (k == "medium_max") {
        if (value != 64 && value != 128 && value != 256 && value != 512) return QZGPU_BAD_PARAMETER;
        each([&](Tune& t) { t.medium_max = (int)value; });
    } else if (k == "ruler_stride_log2") {
        if (value < 3 || value > 12) return QZGPU_BAD_PARAMETER;
        each([&](Tune& t) { t.ruler_log2 = (int)value; });
    } else if (k == "big_tile") {
        if (value != 2048 && value != 4096 && value != 8192) return QZGPU_BAD_PARAMETER;
        each([&](Tune& t) { t.big_tile = (int)value; });
    } else if (k == "radix_first_bits") {
        if (value < 8 || value > 11) return QZGPU_BAD_PARAMETER;
        each([&](Tune& t) { t.first_digit_max = (int)value; });
    } else if (k == "round_pipeline") {
        if (value < 0 || value > 1) return QZGPU_BAD_PARAMETER;
        each([&](Tune& t) { t.round_pipeline = (int)value; });
    } else if (k == "split_lookback") {
        if (value < 0 || value > 1) return QZGPU_BAD_PARAMETER;
        each([&](Tune& t) { t.split_lookback = (int)value; });
    } else if (k == "rank_mode") {
        if (value < 0 || value > 2) return QZGPU_BAD_PARAMETER;
        each([&](Tune& t) { t.rank_mode = (int)value; });
    } else if (k == "early_counts") {
        if (value < 0 || value > 1) return QZGPU_BAD_PARAMETER;
        each([&](Tune& t) { t.early_counts = (int)value; });
    } else if (k == "pass0_bulk") {
        if (value < 0 || value > 1) return QZGPU_BAD_PARAMETER;
        each([&](Tune& t) { t.pass0_bulk = (int)value; });
    } else if (k == "lookback_test") {
        if (value < 0 || value > 2) return QZGPU_BAD_PARAMETER;
        each([&](Tune& t) { t.lookback_test = (int)value; });
    } else {
        return QZGPU_BAD_PARAMETER;
    }
    return QZGPU_NO_ERROR;
}

long long qzgpu_storage_get_param(const qzgpu_storage* storage, const char* name) {
    if (!storage || !name || storage->lanes.empty()) return QZGPU_BAD_PARAMETER;
    std::string k(name);
    const Tune& t = storage->lanes[0]->tune;
    if (k == "fwd_sub_bytes") return storage->fwd_sub_bytes;
    if (k == "inv_sub_bytes") return storage->inv_sub_bytes;
    if (k == "big_ctas_per_sm") return t.big_ctas_per_sm;
    if (k == "tile_ctas_per_sm") return t.tile_ctas_per_sm;
    if (k == "medium_max") return t.medium_max;
    if (k == "ruler_stride_log2") return t.ruler_log2;
    if (k == "big_tile") return t.big_tile;
    if (k == "radix_first_bits") return t.first_digit_max;
    if (k == "round_pipeline") return t.round_pipeline;
    if (k == "split_lookback") return t.split_lookback;
    if (k == "rank_mode") return t.rank_mode;
    if (k == "early_counts") return t.early_counts;
    if (k == "pass0_bulk") return t.pass0_bulk;
    if (k == "lookback_test") return t.lookback_test;
    if (k == "lanes") return (long long)storage->lanes.size();
    return QZGPU_BAD_PARAMETER;
}

int qzgpu_storage_round_counts(const qzgpu_storage* storage, long long* active, int max) {
    if (!storage || max < 0 || (max > 0 && !active)) return QZGPU_BAD_PARAMETER;
    int n = (int)storage->rounds_active.size();
    for (int i = 0; i < n && i < max; ++i) active[i] = storage->rounds_active[i];
    return n;
}

int qzgpu_storage_profile(qzgpu_storage* storage, int enable) {
    if (!storage) return QZGPU_BAD_PARAMETER;
    std::lock_guard<std::mutex> lk(storage->mu);
    storage->profile = enable != 0;
    return QZGPU_NO_ERROR;
}

int qzgpu_storage_profile_only(qzgpu_storage* storage, const char* name) {
    if (!storage) return QZGPU_BAD_PARAMETER;
    std::lock_guard<std::mutex> lk(storage->mu);
    storage->profile_only = name ? name : "";
    return QZGPU_NO_ERROR;
}

int qzgpu_storage_profile_read(qzgpu_storage* storage, qzgpu_kernel_time* out, int max, int reset) {
    if (!storage || max < 0 || (max > 0 && !out)) return QZGPU_BAD_PARAMETER;
    std::lock_guard<std::mutex> lk(storage->mu);
    std::vector<std::pair<std::string, Storage::ProfAgg>> v(storage->prof.begin(), storage->prof.end());
    std::sort(v.begin(), v.end(), [](const auto& x, const auto& y) { return x.second.ms > y.second.ms; });
    for (int i = 0; i < max && i < (int)v.size(); ++i) {
        memset(out[i].name, 0, sizeof(out[i].name));
        strncpy(out[i].name, v[i].first.c_str(), sizeof(out[i].name) - 1);
        out[i].launches = v[i].second.launches;
        out[i].ms = v[i].second.ms;
        out[i].alg_bytes = v[i].second.bytes;
    }
    int n = (int)v.size();
    if (reset) storage->prof.clear();
    return n;
}

int qzgpu_storage_last_stats(const qzgpu_storage* storage, qzgpu_stats* out) {
    if (!storage || !out) return QZGPU_BAD_PARAMETER;
    *out = storage->stats;
    return QZGPU_NO_ERROR;
}

}  // extern "C"
