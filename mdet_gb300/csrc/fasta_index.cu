// fasta_index.cu -- FASTA ingest on the device: the reference reader's record
// split (cuda/Cuda2.cu:1486-1553) over the file's bytes in HBM, so that a
// caller can go from the raw file to TNF rows without a host pass over it.
//
// Record rules (the reference's loop read sequentially): a '>' starts a record
// wherever it stands, except inside the name line of the record before it;
// so the record starts are exactly the first '>' of each line.  The name is
// the rest of that line cut at its first space; the sequence view runs from
// after the name line's newline to the next record's '>' (or the end), inner
// newlines kept, one trailing newline dropped; the size is the view's bytes
// before that drop minus its newlines.  A name line that reaches the end of
// the buffer without a newline is not a record.
//
// Pass 1 (k_fa_starts) reads every byte once in 16-byte loads; a thread that
// sees a '>' settles whether it is the first of its line from its own 16 bytes
// or, when the line began in an earlier chunk, by walking back to the line's
// previous '\n' or '>'.  Starts are appended with an atomic (they are rare:
// one per record) and sorted.  Pass 2 (k_fa_records) gives each record a warp:
// it finds the name line's newline and first space with ballots over 32-byte
// windows, then counts the newlines of the sequence view with 16-byte loads
// (the view's bytes are read once more).  A scan of the size-class flags
// places the records with size >= min_contig in file order.
#include <cstring>

#include <cub/cub.cuh>

#include "common.cuh"

namespace {

constexpr uint64_t kNone = ~0ull;

__device__ __forceinline__ unsigned char byte_of(const uint4& q, int j) {
    const uint32_t w = j < 4 ? q.x : j < 8 ? q.y : j < 12 ? q.z : q.w;
    return (unsigned char)(w >> (8 * (j & 3)));
}

// Is the '>' whose line reaches back before position p (exclusive) the first
// of its line?  Walks back to the previous '\n' (yes) or '>' (no); the
// buffer's start is a line start.
__device__ bool line_has_no_gt_before(const unsigned char* __restrict__ b, uint64_t p) {
    while (p > 0) {
        const unsigned char c = b[--p];
        if (c == '\n') return true;
        if (c == '>') return false;
    }
    return true;
}

// The '>' bytes of one 16-byte chunk at base: appends the record starts.
__device__ __forceinline__ void chunk_starts(const unsigned char* __restrict__ b, uint64_t base, const uint4& q,
                                             uint64_t* __restrict__ starts, uint64_t cap,
                                             unsigned long long* __restrict__ count) {
    const uint32_t any = __vcmpeq4(q.x, 0x3E3E3E3Eu) | __vcmpeq4(q.y, 0x3E3E3E3Eu) | __vcmpeq4(q.z, 0x3E3E3E3Eu) |
                         __vcmpeq4(q.w, 0x3E3E3E3Eu);
    if (!any) return;
    // state carried left to right through the chunk: 1 = a line start (no '>'
    // since the last '\n'), 0 = a '>' already on this line, 2 = not known yet
    // (the line began before this chunk)
    int state = 2;
    for (int j = 0; j < 16; ++j) {
        const unsigned char ch = byte_of(q, j);
        if (ch == '\n') {
            state = 1;
        } else if (ch == '>') {
            if (state == 2) state = line_has_no_gt_before(b, base) ? 1 : 0;
            if (state == 1) {
                const unsigned long long pos = atomicAdd(count, 1ull);
                if (pos < cap) starts[pos] = base + j;
            }
            state = 0;
        }
    }
}

// Four chunks per thread and round, their loads issued together.
__global__ void k_fa_starts(const unsigned char* __restrict__ b, uint64_t nbytes, uint64_t* __restrict__ starts,
                            uint64_t cap, unsigned long long* __restrict__ count) {
    const uint64_t nfull = nbytes / 16;
    const uint64_t G = (uint64_t)gridDim.x * blockDim.x;
    const uint64_t t = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x;
    const uint4* b4 = reinterpret_cast<const uint4*>(b);
    for (uint64_t c = t; c < nfull; c += 4 * G) {
        uint4 q[4];
#pragma unroll
        for (int u = 0; u < 4; ++u) q[u] = c + u * G < nfull ? __ldg(b4 + c + u * G) : make_uint4(0, 0, 0, 0);
#pragma unroll
        for (int u = 0; u < 4; ++u)
            if (c + u * G < nfull) chunk_starts(b, (c + u * G) * 16, q[u], starts, cap, count);
    }
    if (t == 0 && nbytes % 16) {  // the ragged last chunk
        const uint64_t base = nfull * 16;
        uint32_t w[4] = {0, 0, 0, 0};
        for (uint64_t j = 0; base + j < nbytes; ++j) w[j >> 2] |= (uint32_t)b[base + j] << (8 * (j & 3));
        chunk_starts(b, base, make_uint4(w[0], w[1], w[2], w[3]), starts, cap, count);
    }
}

struct RecArgs {
    const unsigned char* b;
    uint64_t nbytes;
    const uint64_t* starts;
    uint64_t nr;
    uint64_t min_contig;
    uint64_t* off;       // per record: sequence view offset
    uint64_t* len;       // view length
    uint64_t* size;      // bases
    uint64_t* name_off;
    uint32_t* name_len;
    uint32_t* large;     // 1: a record with size >= min_contig
    unsigned long long* n_valid;
    unsigned long long* n_small;
};

// A warp per record.
__global__ void k_fa_records(RecArgs p) {
    const uint32_t lane = threadIdx.x & 31;
    const uint64_t nw = (uint64_t)gridDim.x * (blockDim.x >> 5);
    for (uint64_t r = (blockIdx.x * (uint64_t)blockDim.x + threadIdx.x) >> 5; r < p.nr; r += nw) {
        const uint64_t g = p.starts[r];
        const uint64_t nx = r + 1 < p.nr ? p.starts[r + 1] : p.nbytes;
        // name line: its newline h and the first space before it
        uint64_t h = kNone, sp = kNone;
        for (uint64_t q0 = g + 1; q0 < nx; q0 += 32) {
            const uint64_t q = q0 + lane;
            const unsigned char ch = q < nx ? p.b[q] : 0;
            const uint32_t nlm = __ballot_sync(0xffffffffu, ch == '\n');
            const uint32_t spm = __ballot_sync(0xffffffffu, ch == ' ');
            const uint32_t lim = nlm ? (nlm & (0u - nlm)) - 1u : 0xffffffffu;  // lanes before the newline
            if (sp == kNone && (spm & lim)) sp = q0 + __ffs(spm & lim) - 1;
            if (nlm) {
                h = q0 + __ffs(nlm) - 1;
                break;
            }
        }
        if (h == kNone) {  // the name line runs into the end of the buffer: no record
            if (lane == 0) p.large[r] = 0;
            continue;
        }
        const uint64_t s0 = h + 1, s1 = nx;
        // newlines of the view [s0, s1): ragged head and tail by bytes, the
        // aligned middle by 16-byte loads
        uint64_t a0 = (s0 + 15) & ~15ull, a1 = s1 & ~15ull;
        if (a0 > s1) a0 = s1;
        if (a1 < a0) a1 = a0;
        uint32_t nl = 0;
        if (s0 + lane < a0) nl += p.b[s0 + lane] == '\n';
        if (a1 + lane < s1) nl += p.b[a1 + lane] == '\n';
        // four 16-byte loads per lane in flight
        for (uint64_t c = a0 + 16 * (uint64_t)lane; c < a1; c += 4 * 16 * 32) {
            uint4 q[4];
#pragma unroll
            for (int u = 0; u < 4; ++u) {
                const uint64_t cu = c + (uint64_t)u * 16 * 32;
                q[u] = cu < a1 ? __ldg(reinterpret_cast<const uint4*>(p.b + cu)) : make_uint4(0, 0, 0, 0);
            }
#pragma unroll
            for (int u = 0; u < 4; ++u)
                nl += (__popc(__vcmpeq4(q[u].x, 0x0A0A0A0Au)) + __popc(__vcmpeq4(q[u].y, 0x0A0A0A0Au)) +
                       __popc(__vcmpeq4(q[u].z, 0x0A0A0A0Au)) + __popc(__vcmpeq4(q[u].w, 0x0A0A0A0Au))) >>
                      3;
        }
#pragma unroll
        for (int d = 16; d; d >>= 1) nl += __shfl_xor_sync(0xffffffffu, nl, d);
        if (lane == 0) {
            uint64_t view = s1 - s0;
            const uint64_t sz = view - nl;
            if (view > 0 && p.b[s1 - 1] == '\n') --view;
            p.off[r] = s0;
            p.len[r] = view;
            p.size[r] = sz;
            p.name_off[r] = g + 1;
            p.name_len[r] = (uint32_t)((sp != kNone ? sp : h) - (g + 1));
            p.large[r] = sz >= p.min_contig ? 1u : 0u;
            atomicAdd(p.n_valid, 1ull);
            if (sz < p.min_contig && sz >= 1000) atomicAdd(p.n_small, 1ull);
        }
    }
}

struct EmitArgs {
    uint64_t nr, cap;
    const uint32_t* large;
    const uint32_t* dst;
    const uint64_t *off, *len, *size, *name_off;
    const uint32_t* name_len;
    uint64_t *o_off, *o_len, *o_size, *o_name_off;
    double* o_log_size;
    uint32_t* o_name_len;
};

__global__ void k_fa_emit(EmitArgs p) {
    for (uint64_t r = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; r < p.nr;
         r += (uint64_t)gridDim.x * blockDim.x) {
        if (!p.large[r]) continue;
        const uint64_t k = p.dst[r];
        if (k >= p.cap) continue;
        p.o_off[k] = p.off[r];
        p.o_len[k] = p.len[r];
        const uint64_t sz = p.size[r];
        if (p.o_size) p.o_size[k] = sz;
        // log10(min(size, 500000)) (cuda/Cuda2.cu:1535)
        if (p.o_log_size) p.o_log_size[k] = log10((double)(sz < 500000 ? sz : 500000));
        if (p.o_name_off) p.o_name_off[k] = p.name_off[r];
        if (p.o_name_len) p.o_name_len[k] = p.name_len[r];
    }
}

unsigned grid_for(mdet_ctx* ctx, uint64_t items, unsigned block) {
    const uint64_t want = (items + block - 1) / block, cap = (uint64_t)ctx->num_sms * 16;
    return (unsigned)(want < 1 ? 1 : (want < cap ? want : cap));
}

struct FastaOut {
    uint64_t *off, *len, *size, *name_off;
    double* log_size;
    uint32_t* name_len;
};

int index_core(mdet_ctx* ctx, const char* d_bytes, uint64_t nbytes, uint64_t min_contig, uint64_t capacity,
               const FastaOut& o, mdet_fasta_stats* st) {
    cudaStream_t s = ctx->stream;
    const unsigned char* b = (const unsigned char*)d_bytes;
    unsigned long long* cnt = (unsigned long long*)ctx_scratch(ctx, "fa.cnt", 3 * 8);
    if (!cnt) return MDET_ERR_NOMEM;
    // pass 1: record starts (sized by a guess, redone once at the exact count)
    uint64_t cap = nbytes / 2048 + 4096;
    DevBuf& sb = ctx->bufs["fa.starts"];
    if (sb.cap / 8 > cap) cap = sb.cap / 8;
    unsigned long long h_cnt[3] = {0, 0, 0};
    uint64_t* starts = nullptr;
    for (int attempt = 0; attempt < 2; ++attempt) {
        starts = (uint64_t*)ctx_scratch(ctx, "fa.starts", cap * 8);
        if (!starts) return MDET_ERR_NOMEM;
        cap = ctx->bufs["fa.starts"].cap / 8;
        MDET_CUDA(ctx, cudaMemsetAsync(cnt, 0, 3 * 8, s));
        ctx_timer_begin(ctx, "k_fa_starts");
        k_fa_starts<<<grid_for(ctx, (nbytes / 16 + 3) / 4, 256), 256, 0, s>>>(b, nbytes, starts, cap, cnt);
        ctx_timer_end(ctx, "k_fa_starts");
        MDET_LAUNCHED(ctx, "k_fa_starts");
        MDET_CUDA(ctx, cudaMemcpyAsync(h_cnt, cnt, 8, cudaMemcpyDeviceToHost, s));
        MDET_CUDA(ctx, cudaStreamSynchronize(s));
        if (h_cnt[0] <= cap) break;
        cap = h_cnt[0];
    }
    const uint64_t nr = h_cnt[0];
    if (nr >= (1ull << 31)) return ctx_fail(ctx, MDET_ERR_INVALID, "too many FASTA records (%llu)", (unsigned long long)nr);
    st->n_records = st->n_large = st->n_small = 0;
    if (nr == 0) return MDET_OK;
    uint64_t* sorted = (uint64_t*)ctx_scratch(ctx, "fa.sorted", nr * 8);
    uint64_t* r_off = (uint64_t*)ctx_scratch(ctx, "fa.off", nr * 8);
    uint64_t* r_len = (uint64_t*)ctx_scratch(ctx, "fa.len", nr * 8);
    uint64_t* r_size = (uint64_t*)ctx_scratch(ctx, "fa.size", nr * 8);
    uint64_t* r_noff = (uint64_t*)ctx_scratch(ctx, "fa.noff", nr * 8);
    uint32_t* r_nlen = (uint32_t*)ctx_scratch(ctx, "fa.nlen", nr * 4);
    uint32_t* large = (uint32_t*)ctx_scratch(ctx, "fa.large", (nr + 1) * 4);
    uint32_t* dst = (uint32_t*)ctx_scratch(ctx, "fa.dst", (nr + 1) * 4);
    if (!sorted || !r_off || !r_len || !r_size || !r_noff || !r_nlen || !large || !dst) return MDET_ERR_NOMEM;
    int bits = 1;
    while (bits < 64 && (nbytes >> bits)) ++bits;
    size_t t1 = 0, t2 = 0;
    MDET_CUDA(ctx, cub::DeviceRadixSort::SortKeys(nullptr, t1, starts, sorted, (int)nr, 0, bits, s));
    MDET_CUDA(ctx, cub::DeviceScan::ExclusiveSum(nullptr, t2, large, dst, (int)nr + 1, s));
    void* tmp = ctx_scratch(ctx, "fa.cubtmp", t1 > t2 ? t1 : t2);
    if (!tmp) return MDET_ERR_NOMEM;
    MDET_CUDA(ctx, cub::DeviceRadixSort::SortKeys(tmp, t1, starts, sorted, (int)nr, 0, bits, s));

    RecArgs ra{b, nbytes, sorted, nr, min_contig, r_off, r_len, r_size, r_noff, r_nlen, large, cnt + 1, cnt + 2};
    ctx_timer_begin(ctx, "k_fa_records");
    k_fa_records<<<grid_for(ctx, nr * 32, 256), 256, 0, s>>>(ra);
    ctx_timer_end(ctx, "k_fa_records");
    MDET_LAUNCHED(ctx, "k_fa_records");
    // the scan runs over nr + 1 flags so that dst[nr] is the count
    MDET_CUDA(ctx, cudaMemsetAsync(large + nr, 0, 4, s));
    MDET_CUDA(ctx, cub::DeviceScan::ExclusiveSum(tmp, t2, large, dst, (int)nr + 1, s));
    EmitArgs ea{nr, capacity, large, dst, r_off, r_len, r_size, r_noff, r_nlen,
                o.off, o.len, o.size, o.name_off, o.log_size, o.name_len};
    k_fa_emit<<<grid_for(ctx, nr, 256), 256, 0, s>>>(ea);
    MDET_LAUNCHED(ctx, "k_fa_emit");
    uint32_t nlarge = 0;
    MDET_CUDA(ctx, cudaMemcpyAsync(&nlarge, dst + nr, 4, cudaMemcpyDeviceToHost, s));
    MDET_CUDA(ctx, cudaMemcpyAsync(h_cnt + 1, cnt + 1, 16, cudaMemcpyDeviceToHost, s));
    MDET_CUDA(ctx, cudaStreamSynchronize(s));
    st->n_records = h_cnt[1];
    st->n_large = nlarge;
    st->n_small = h_cnt[2];
    if (nlarge > capacity)
        return ctx_fail(ctx, MDET_ERR_CAPACITY, "%llu contigs of at least %llu bases, capacity %llu",
                        (unsigned long long)nlarge, (unsigned long long)min_contig, (unsigned long long)capacity);
    return MDET_OK;
}

}  // namespace

extern "C" {

int mdet_fasta_index_dev(mdet_ctx* ctx, const char* d_bytes, uint64_t nbytes, uint64_t min_contig,
                         uint64_t capacity, uint64_t* d_seq_off, uint64_t* d_seq_len, uint64_t* d_size,
                         double* d_log_size, uint64_t* d_name_off, uint32_t* d_name_len, mdet_fasta_stats* stats) {
    if (!ctx || !stats) return MDET_ERR_INVALID;
    MDET_CUDA(ctx, cudaSetDevice(ctx->device));
    ctx->launches = 0;
    memset(stats, 0, sizeof(*stats));
    if (nbytes == 0) return MDET_OK;
    if (!d_bytes) return ctx_fail(ctx, MDET_ERR_INVALID, "null pointer");
    if (((uintptr_t)d_bytes & 15) != 0) return ctx_fail(ctx, MDET_ERR_INVALID, "FASTA buffer must be 16-byte aligned");
    if (capacity && (!d_seq_off || !d_seq_len)) return ctx_fail(ctx, MDET_ERR_INVALID, "null output pointer");
    cudaEvent_t e0, e1;
    cudaEventCreate(&e0);
    cudaEventCreate(&e1);
    cudaEventRecord(e0, ctx->stream);
    const FastaOut o{d_seq_off, d_seq_len, d_size, d_name_off, d_log_size, d_name_len};
    int rc = index_core(ctx, d_bytes, nbytes, min_contig, capacity, o, stats);
    cudaEventRecord(e1, ctx->stream);
    float ms = 0;
    cudaEventSynchronize(e1);
    cudaEventElapsedTime(&ms, e0, e1);
    stats->ms_total = ms;
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    return rc;
}

int mdet_fasta_index(mdet_ctx* ctx, const char* bytes, uint64_t nbytes, uint64_t min_contig, uint64_t capacity,
                     uint64_t* seq_off, uint64_t* seq_len, uint64_t* size, double* log_size, uint64_t* name_off,
                     uint32_t* name_len, mdet_fasta_stats* stats) {
    if (!ctx || !stats) return MDET_ERR_INVALID;
    MDET_CUDA(ctx, cudaSetDevice(ctx->device));
    memset(stats, 0, sizeof(*stats));
    if (nbytes == 0) return MDET_OK;
    if (!bytes) return ctx_fail(ctx, MDET_ERR_INVALID, "null pointer");
    cudaStream_t s = ctx->stream;
    char* d_bytes = (char*)ctx_scratch(ctx, "io.bytes", nbytes + 64);
    const uint64_t c = capacity ? capacity : 1;
    uint64_t* d_off = (uint64_t*)ctx_scratch(ctx, "io.fa_off", c * 8);
    uint64_t* d_len = (uint64_t*)ctx_scratch(ctx, "io.fa_len", c * 8);
    uint64_t* d_size = (uint64_t*)ctx_scratch(ctx, "io.fa_size", c * 8);
    double* d_ls = (double*)ctx_scratch(ctx, "io.fa_ls", c * 8);
    uint64_t* d_noff = (uint64_t*)ctx_scratch(ctx, "io.fa_noff", c * 8);
    uint32_t* d_nlen = (uint32_t*)ctx_scratch(ctx, "io.fa_nlen", c * 4);
    if (!d_bytes || !d_off || !d_len || !d_size || !d_ls || !d_noff || !d_nlen) return MDET_ERR_NOMEM;
    MDET_CUDA(ctx, cudaMemcpyAsync(d_bytes, bytes, nbytes, cudaMemcpyHostToDevice, s));
    int rc = mdet_fasta_index_dev(ctx, d_bytes, nbytes, min_contig, capacity, d_off, d_len, d_size, d_ls, d_noff,
                                  d_nlen, stats);
    if (rc != MDET_OK) return rc;
    const uint64_t k = stats->n_large;
    if (k) {
        if (seq_off) MDET_CUDA(ctx, cudaMemcpyAsync(seq_off, d_off, k * 8, cudaMemcpyDeviceToHost, s));
        if (seq_len) MDET_CUDA(ctx, cudaMemcpyAsync(seq_len, d_len, k * 8, cudaMemcpyDeviceToHost, s));
        if (size) MDET_CUDA(ctx, cudaMemcpyAsync(size, d_size, k * 8, cudaMemcpyDeviceToHost, s));
        if (log_size) MDET_CUDA(ctx, cudaMemcpyAsync(log_size, d_ls, k * 8, cudaMemcpyDeviceToHost, s));
        if (name_off) MDET_CUDA(ctx, cudaMemcpyAsync(name_off, d_noff, k * 8, cudaMemcpyDeviceToHost, s));
        if (name_len) MDET_CUDA(ctx, cudaMemcpyAsync(name_len, d_nlen, k * 4, cudaMemcpyDeviceToHost, s));
    }
    MDET_CUDA(ctx, cudaStreamSynchronize(s));
    return MDET_OK;
}

}  // extern "C"
