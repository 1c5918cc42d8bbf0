// Stream building on the device: FASTQ text -> qz's header, sequence and
// quality streams for its default lossless BSC path (sm_103a, byte work).
//
// Replaces records_to_streams (crates/qz-lib/src/compression/mod.rs:270-325)
// with the FASTQ reader that feeds it (io/fastq.rs:135-200) and
// detect_const_lengths (mod.rs:329-354); the quality packing is
// pack_qualities with binning None (compression/columnar.rs:104-134).
//
//   1. k_nl_count / k_nl_write: the line ends of the text, in order (64 KB
//      tiles, one count pass, a scan of the tile counts, one write pass);
//   2. k_records: per record, its four lines: trimmed id / sequence / quality
//      lengths, the '+' check and the length check (first failing record kept);
//   3. header offsets by a scan of varint + id sizes; sequence and quality
//      offsets are closed-form when the lengths are constant;
//   4. k_fill: one warp per record writes its varint(s), id, bases and packed
//      qualities (each packed byte from the two quality values it covers).
#include <mutex>

#include "engine.h"
#include "scan.cuh"

namespace qz {

namespace {

constexpr int kStTile = 65536;                    // text bytes per tile
constexpr int kStPerThread = kStTile / kThreads;  // 256 bytes per thread

// bytes of write_varint(v) (7 bits per byte)
__device__ __forceinline__ int vlen(uint32_t v) {
    return v < (1u << 7) ? 1 : v < (1u << 14) ? 2 : v < (1u << 21) ? 3 : v < (1u << 28) ? 4 : 5;
}

// Newlines among the 256 bytes a thread owns (16-byte loads when the run is
// inside the text; the text copy is 16-byte aligned).
__device__ __forceinline__ uint32_t nl_bits16(uint4 v) {
    // one bit per byte equal to '\n', in byte order
    uint32_t m = 0;
    const uint32_t w[4] = {v.x, v.y, v.z, v.w};
#pragma unroll
    for (int q = 0; q < 4; ++q) {
#pragma unroll
        for (int b = 0; b < 4; ++b) m |= (uint32_t)(((w[q] >> (8 * b)) & 0xffu) == '\n') << (4 * q + b);
    }
    return m;
}

__device__ __forceinline__ uint32_t count_nl(const uint8_t* __restrict__ text, long long n, long long base) {
    uint32_t c = 0;
    if (base + kStPerThread <= n) {
        const uint4* p = reinterpret_cast<const uint4*>(text + base);
#pragma unroll 4
        for (int k = 0; k < kStPerThread / 16; ++k) c += __popc(nl_bits16(__ldg(p + k)));
    } else {
        for (int k = 0; k < kStPerThread; ++k) {
            const long long x = base + k;
            if (x < n) c += text[x] == '\n';
        }
    }
    return c;
}

__global__ void __launch_bounds__(kThreads) k_nl_count(const uint8_t* __restrict__ text, long long n,
                                                       uint32_t* __restrict__ cnt) {
    __shared__ uint32_t sh[kWarps + 1];
    const long long base = (long long)blockIdx.x * kStTile + (long long)threadIdx.x * kStPerThread;
    const uint32_t c = count_nl(text, n, base);
    uint32_t tot;
    block_excl_sum(c, sh, &tot);
    if (threadIdx.x == 0) cnt[blockIdx.x] = tot;
}

__global__ void __launch_bounds__(kThreads) k_nl_write(const uint8_t* __restrict__ text, long long n,
                                                       const uint32_t* __restrict__ tbase, int* __restrict__ line_end) {
    __shared__ uint32_t sh[kWarps + 1];
    const long long base = (long long)blockIdx.x * kStTile + (long long)threadIdx.x * kStPerThread;
    const uint32_t c = count_nl(text, n, base);
    uint32_t tot;
    uint32_t at = tbase[blockIdx.x] + block_excl_sum(c, sh, &tot);
    if (!c) return;
    if (base + kStPerThread <= n) {
        const uint4* p = reinterpret_cast<const uint4*>(text + base);
        for (int k = 0; k < kStPerThread / 16; ++k) {
            uint32_t m = nl_bits16(__ldg(p + k));
            while (m) {
                line_end[at++] = (int)(base + 16 * k + __ffs(m) - 1);
                m &= m - 1;
            }
        }
    } else {
        for (int k = 0; k < kStPerThread; ++k) {
            const long long x = base + k;
            if (x < n && text[x] == '\n') line_end[at++] = (int)x;
        }
    }
}

struct RecArgs {
    const uint8_t* text;
    const int* line_end;  // end (exclusive) of each line: its '\n', or n for a final line without one
    long long records;
    int* id_len;
    int* seq_len;
    int* stats;           // [0] min seq len, [1] max seq len, [2] min qual len, [3] max qual len, [4] first bad record
};

__device__ __forceinline__ int line_start(const int* le, long long k) { return k == 0 ? 0 : le[k - 1] + 1; }

// Trimmed length: trailing '\r' dropped (a line never holds '\n').
__device__ __forceinline__ int trimmed(const uint8_t* text, int s, int e) {
    while (e > s && text[e - 1] == '\r') --e;
    return e - s;
}

__global__ void __launch_bounds__(kThreads) k_records(RecArgs a) {
    for (long long r = (long long)blockIdx.x * kThreads + threadIdx.x; r < a.records;
         r += (long long)gridDim.x * kThreads) {
        const long long l0 = 4 * r;
        const int s0 = line_start(a.line_end, l0), e0 = a.line_end[l0];
        const int s1 = e0 + 1, e1 = a.line_end[l0 + 1];
        const int s2 = e1 + 1, e2 = a.line_end[l0 + 2];
        const int s3 = e2 + 1, e3 = a.line_end[l0 + 3];
        const int il = trimmed(a.text, s0, e0);
        const int sl = trimmed(a.text, s1, e1);
        const int ql = trimmed(a.text, s3, e3);
        // the separator line must start with '+' (an empty line starts with its '\n')
        const bool sep_ok = e2 > s2 && a.text[s2] == '+';
        if (!sep_ok || ql != sl) atomicMin(&a.stats[4], (int)r);
        a.id_len[r] = il;
        a.seq_len[r] = sl;
        atomicMin(&a.stats[0], sl);
        atomicMax(&a.stats[1], sl);
        atomicMin(&a.stats[2], ql);
        atomicMax(&a.stats[3], ql);
    }
}

__global__ void __launch_bounds__(kThreads) k_hdr_sizes(const int* __restrict__ id_len, long long records,
                                                        uint32_t* __restrict__ sz) {
    for (long long r = (long long)blockIdx.x * kThreads + threadIdx.x; r < records;
         r += (long long)gridDim.x * kThreads)
        sz[r] = (uint32_t)(vlen((uint32_t)id_len[r]) + id_len[r]);
}

__global__ void __launch_bounds__(kThreads) k_var_sizes(const int* __restrict__ seq_len, long long records,
                                                        uint32_t* __restrict__ ssz, uint32_t* __restrict__ qsz) {
    for (long long r = (long long)blockIdx.x * kThreads + threadIdx.x; r < records;
         r += (long long)gridDim.x * kThreads) {
        const uint32_t L = (uint32_t)seq_len[r];
        ssz[r] = (uint32_t)vlen(L) + L;
        qsz[r] = (uint32_t)vlen(L) + (uint32_t)((7ull * L + 7) / 8);
    }
}

struct FillArgs {
    const uint8_t* text;
    const int* line_end;
    long long records;
    const int* id_len;
    const int* seq_len;
    const uint32_t* hoff;  // header offset per record
    const uint32_t* soff;  // sequence / quality offsets when lengths vary (else null)
    const uint32_t* qoff;
    int cseq;              // constant length, or 0
    uint8_t* hdr;
    uint8_t* seq;
    uint8_t* qual;
};

__device__ __forceinline__ int put_varint(uint8_t* out, uint32_t v) {
    int k = 0;
    while (v >= 0x80) {
        out[k++] = (uint8_t)((v & 0x7f) | 0x80);
        v >>= 7;
    }
    out[k++] = (uint8_t)v;
    return k;
}

__device__ __forceinline__ uint32_t enc7(uint8_t q) { return q < 33 ? 0u : min((uint32_t)(q - 33), 127u); }

__global__ void __launch_bounds__(kThreads) k_fill(FillArgs a) {
    const int ln = (int)lane_id();
    const long long nw = (long long)gridDim.x * kWarps;
    for (long long r = (long long)blockIdx.x * kWarps + warp_id(); r < a.records; r += nw) {
        const long long l0 = 4 * r;
        const int s0 = line_start(a.line_end, l0);
        const int s1 = a.line_end[l0] + 1;
        const int s3 = a.line_end[l0 + 2] + 1;
        const int il = a.id_len[r], L = a.seq_len[r];
        // header: varint + id
        uint8_t* h = a.hdr + a.hoff[r];
        int hv = vlen((uint32_t)il);
        if (ln == 0) put_varint(h, (uint32_t)il);
        for (int k = ln; k < il; k += 32) h[hv + k] = a.text[s0 + k];
        // sequence: (varint) + bases
        const long long packed = (7LL * L + 7) / 8;
        uint8_t* sq;
        uint8_t* qp;
        if (a.cseq) {
            sq = a.seq + (long long)r * L;
            qp = a.qual + (long long)r * packed;
        } else {
            sq = a.seq + a.soff[r];
            qp = a.qual + a.qoff[r];
            const int v = vlen((uint32_t)L);
            if (ln == 0) {
                put_varint(sq, (uint32_t)L);
                put_varint(qp, (uint32_t)L);
            }
            sq += v;
            qp += v;
        }
        for (int k = ln; k < L; k += 32) sq[k] = a.text[s1 + k];
        // qualities: output byte j holds bits 8j .. 8j+7 of the 7-bit values
        for (long long j = ln; j < packed; j += 32) {
            const long long bit = 8 * j, v = bit / 7;
            const int sh = (int)(bit % 7);
            // value v supplies 7 - sh bits, value v + 1 the rest (sh <= 6)
            uint32_t w = enc7(a.text[s3 + v]) >> sh;
            if (v + 1 < L) w |= enc7(a.text[s3 + v + 1]) << (7 - sh);
            qp[j] = (uint8_t)w;
        }
    }
}

// Device scratch of the stream builder, grown on demand; one call at a time.
struct StreamCtx {
    std::mutex mu;
    int device = -1;
    cudaStream_t st = nullptr;
    long long cap = 0;       // text bytes
    char* base = nullptr;    // the one allocation the arrays below are carved from
    uint8_t* text = nullptr;
    uint32_t* tcnt = nullptr;
    uint32_t* tbase = nullptr;
    int* line_end = nullptr;
    int* id_len = nullptr;
    int* seq_len = nullptr;
    uint32_t* hsz = nullptr;
    uint32_t* hoff = nullptr;
    uint32_t* ssz = nullptr;
    uint32_t* soff = nullptr;
    uint32_t* qsz = nullptr;
    uint32_t* qoff = nullptr;
    uint8_t* out = nullptr;  // three streams back to back
    long long out_cap = 0;
    int* stats = nullptr;
    int* pin = nullptr;
    Storage scan;            // only its scan partials are used
};

StreamCtx& ctx() {
    static StreamCtx c;
    return c;
}

int grow(StreamCtx& c, long long n) {
    if (n <= c.cap && c.st) return QZGPU_NO_ERROR;
    long long cap = std::max<long long>(n, 1 << 20);
    cudaFree(c.base);
    c.base = nullptr;
    c.cap = 0;
    const long long tiles = cap / kStTile + 2;
    const long long lines = cap + 2;
    const long long recs = cap / 4 + 2;
    const long long outb = 3 * (cap + 5 * recs) + 64;
    size_t bytes = 0;
    auto take = [&](size_t b) {
        size_t at = bytes;
        bytes += (b + 255) / 256 * 256;
        return at;
    };
    size_t o_text = take(cap + 16), o_tc = take(4 * tiles), o_tb = take(4 * tiles), o_le = take(4 * lines),
           o_il = take(4 * recs), o_sl = take(4 * recs), o_hs = take(4 * recs), o_ho = take(4 * recs),
           o_ss = take(4 * recs), o_so = take(4 * recs), o_qs = take(4 * recs), o_qo = take(4 * recs),
           o_out = take(outb), o_st = take(64), o_part = take(4 * 1024);
    char* base = nullptr;
    cudaError_t e = cudaMalloc(&base, bytes);
    if (e != cudaSuccess) return map_cuda_error(e);
    c.base = base;
    c.text = reinterpret_cast<uint8_t*>(base + o_text);
    c.tcnt = reinterpret_cast<uint32_t*>(base + o_tc);
    c.tbase = reinterpret_cast<uint32_t*>(base + o_tb);
    c.line_end = reinterpret_cast<int*>(base + o_le);
    c.id_len = reinterpret_cast<int*>(base + o_il);
    c.seq_len = reinterpret_cast<int*>(base + o_sl);
    c.hsz = reinterpret_cast<uint32_t*>(base + o_hs);
    c.hoff = reinterpret_cast<uint32_t*>(base + o_ho);
    c.ssz = reinterpret_cast<uint32_t*>(base + o_ss);
    c.soff = reinterpret_cast<uint32_t*>(base + o_so);
    c.qsz = reinterpret_cast<uint32_t*>(base + o_qs);
    c.qoff = reinterpret_cast<uint32_t*>(base + o_qo);
    c.out = reinterpret_cast<uint8_t*>(base + o_out);
    c.out_cap = outb;
    c.stats = reinterpret_cast<int*>(base + o_st);
    c.scan.partial = reinterpret_cast<uint32_t*>(base + o_part);
    c.cap = cap;
    if (!c.st) {
        e = cudaStreamCreateWithFlags(&c.st, cudaStreamNonBlocking);
        if (e != cudaSuccess) return map_cuda_error(e);
        e = cudaMallocHost(&c.pin, 64 * sizeof(int));
        if (e != cudaSuccess) return QZGPU_NOT_ENOUGH_MEMORY;
    }
    return QZGPU_NO_ERROR;
}

}  // namespace

}  // namespace qz

extern "C" int qzgpu_fastq_streams(const unsigned char* fastq, long long n, unsigned char* header_out,
                                   long long header_cap, unsigned char* seq_out, long long seq_cap,
                                   unsigned char* qual_out, long long qual_cap, qzgpu_streams_info* info) {
    using namespace qz;
    if (!info || n < 0 || n > 0x7ffffffell || (n > 0 && !fastq)) return QZGPU_BAD_PARAMETER;
    *info = qzgpu_streams_info{0, 0, 0, 0, 0, 0, -1};
    if (n == 0) return QZGPU_NO_ERROR;  // no records: three empty streams
    int dev = 0, sms = 0;
    int rc = device_info(&dev, &sms);
    if (rc) return rc;
    StreamCtx& c = ctx();
    std::lock_guard<std::mutex> lk(c.mu);
    cudaError_t e = cudaSetDevice(dev);
    if (e != cudaSuccess) return map_cuda_error(e);
    rc = grow(c, n);
    if (rc) return rc;
    const cudaStream_t st = c.st;
    const int tiles = (int)((n + kStTile - 1) / kStTile);
    auto fail = [](cudaError_t err) { return map_cuda_error(err); };
    if ((e = cudaMemcpyAsync(c.text, fastq, (size_t)n, cudaMemcpyHostToDevice, st)) != cudaSuccess) return fail(e);
    // ---- line ends
    k_nl_count<<<tiles, kThreads, 0, st>>>(c.text, n, c.tcnt);
    scan_exclusive(&c.scan, c.tcnt, c.tbase, tiles, nullptr, reinterpret_cast<uint32_t*>(c.stats + 8), st);
    k_nl_write<<<tiles, kThreads, 0, st>>>(c.text, n, c.tbase, c.line_end);
    if ((e = cudaMemcpyAsync(c.pin, c.stats + 8, sizeof(int), cudaMemcpyDeviceToHost, st)) != cudaSuccess)
        return fail(e);
    if ((e = cudaStreamSynchronize(st)) != cudaSuccess) return fail(e);
    long long lines = (unsigned)c.pin[0];
    if (fastq[n - 1] != '\n') {
        // a final line without a newline ends at the end of the text
        c.pin[2] = (int)n;
        if ((e = cudaMemcpyAsync(c.line_end + lines, c.pin + 2, sizeof(int), cudaMemcpyHostToDevice, st)) !=
            cudaSuccess)
            return fail(e);
        ++lines;
    }
    const long long records = lines / 4;
    info->records = records;
    // ---- records
    const int init[8] = {0x7fffffff, -1, 0x7fffffff, -1, 0x7fffffff, 0, 0, 0};
    memcpy(c.pin + 16, init, sizeof(init));
    if ((e = cudaMemcpyAsync(c.stats, c.pin + 16, sizeof(init), cudaMemcpyHostToDevice, st)) != cudaSuccess)
        return fail(e);
    const int rgrid = (int)std::min<long long>((records + kThreads - 1) / kThreads + 1, (long long)sms * 16);
    if (records > 0) k_records<<<rgrid, kThreads, 0, st>>>(RecArgs{c.text, c.line_end, records, c.id_len, c.seq_len, c.stats});
    if ((e = cudaMemcpyAsync(c.pin + 32, c.stats, 5 * sizeof(int), cudaMemcpyDeviceToHost, st)) != cudaSuccess)
        return fail(e);
    if ((e = cudaStreamSynchronize(st)) != cudaSuccess) return fail(e);
    const int* stt = c.pin + 32;
    long long bad = stt[4] == 0x7fffffff ? -1 : stt[4];
    // an input that ends inside a record fails at that record (after any
    // earlier malformed one)
    if (lines % 4 != 0 && (bad < 0 || bad > records)) bad = records;
    if (bad >= 0) {
        info->error_record = bad;
        info->records = bad;
        return QZGPU_DATA_CORRUPT;
    }
    if (records == 0) return QZGPU_NO_ERROR;
    const int cseq = stt[0] == stt[1] ? stt[0] : 0;
    const int cqual = stt[2] == stt[3] ? stt[2] : 0;
    info->const_seq_len = cseq;
    info->const_qual_len = cqual;
    // ---- offsets
    k_hdr_sizes<<<rgrid, kThreads, 0, st>>>(c.id_len, records, c.hsz);
    scan_exclusive(&c.scan, c.hsz, c.hoff, (int)records, nullptr, reinterpret_cast<uint32_t*>(c.stats + 9), st);
    long long sbytes = 0, qbytes = 0;
    if (cseq) {
        sbytes = records * cseq;
        qbytes = records * ((7LL * cseq + 7) / 8);
    } else {
        k_var_sizes<<<rgrid, kThreads, 0, st>>>(c.seq_len, records, c.ssz, c.qsz);
        scan_exclusive(&c.scan, c.ssz, c.soff, (int)records, nullptr, reinterpret_cast<uint32_t*>(c.stats + 10), st);
        scan_exclusive(&c.scan, c.qsz, c.qoff, (int)records, nullptr, reinterpret_cast<uint32_t*>(c.stats + 11), st);
    }
    if ((e = cudaMemcpyAsync(c.pin + 40, c.stats + 9, 3 * sizeof(int), cudaMemcpyDeviceToHost, st)) != cudaSuccess)
        return fail(e);
    if ((e = cudaStreamSynchronize(st)) != cudaSuccess) return fail(e);
    const long long hbytes = (unsigned)c.pin[40];
    if (!cseq) {
        sbytes = (unsigned)c.pin[41];
        qbytes = (unsigned)c.pin[42];
    }
    info->header_bytes = hbytes;
    info->seq_bytes = sbytes;
    info->qual_bytes = qbytes;
    if (header_cap < hbytes || seq_cap < sbytes || qual_cap < qbytes) return QZGPU_BAD_PARAMETER;
    if ((hbytes && !header_out) || (sbytes && !seq_out) || (qbytes && !qual_out)) return QZGPU_BAD_PARAMETER;
    if (hbytes + sbytes + qbytes > c.out_cap) return QZGPU_BAD_PARAMETER;
    // ---- fill and copy out
    FillArgs fa{c.text, c.line_end, records, c.id_len, c.seq_len, c.hoff, cseq ? nullptr : c.soff,
                cseq ? nullptr : c.qoff, cseq, c.out, c.out + hbytes, c.out + hbytes + sbytes};
    const int fgrid = (int)std::min<long long>((records + kWarps - 1) / kWarps, (long long)sms * 16);
    k_fill<<<fgrid, kThreads, 0, st>>>(fa);
    if ((e = cudaGetLastError()) != cudaSuccess) return fail(e);
    if (hbytes && (e = cudaMemcpyAsync(header_out, c.out, (size_t)hbytes, cudaMemcpyDeviceToHost, st)) != cudaSuccess)
        return fail(e);
    if (sbytes &&
        (e = cudaMemcpyAsync(seq_out, c.out + hbytes, (size_t)sbytes, cudaMemcpyDeviceToHost, st)) != cudaSuccess)
        return fail(e);
    if (qbytes && (e = cudaMemcpyAsync(qual_out, c.out + hbytes + sbytes, (size_t)qbytes, cudaMemcpyDeviceToHost,
                                       st)) != cudaSuccess)
        return fail(e);
    if ((e = cudaStreamSynchronize(st)) != cudaSuccess) return fail(e);
    return QZGPU_NO_ERROR;
}
