// pa_input.cu -- the input path around the DP: symbol -> rank conversion, 2-bit
// packing of DNA (host encoder, device encoder and decoder), and the FASTA /
// FASTQ reader.  The kernels are byte streams bound by HBM bandwidth: each
// thread keeps kUnroll 16-byte vector loads in flight per step, grids are a
// multiple of the SM count, and no kernel reads a byte twice.
#include <cuda_runtime.h>

#include <algorithm>
#include <cstdio>
#include <cstring>
#include <string>
#include <vector>

#include "../../include/pairwise_aligner_gb300.h"

namespace pa {

constexpr int kUnroll = 4;     // independent 16-byte loads in flight per thread

// ---------------------------------------------------------------------------------------------
// rank map: the reference's alphabet_rank_map_scalar keeps a 256-entry table (-1 for bytes that
// are not symbols, alphabet_conversion/alphabet_rank_map_scalar.hpp); alphabet_rank_map_simd
// gathers from the same table in SIMD registers (alphabet_rank_map_simd.hpp:31-117).  Here the
// table is held 32 times in shared memory, word w of lane l at [w * 32 + l], so the 32 lanes of a
// warp read 32 different banks whatever bytes they look up.
// ---------------------------------------------------------------------------------------------
__device__ __forceinline__ uint32_t rank4(const uint32_t *tab, int lane, uint32_t w)
{
    uint32_t o = 0;
#pragma unroll
    for (int b = 0; b < 4; ++b) {
        const uint32_t key = (w >> (8 * b)) & 0xffu;
        const uint32_t word = tab[(key >> 2) * 32 + lane];
        o |= ((word >> (8 * (key & 3u))) & 0xffu) << (8 * b);
    }
    return o;
}

__global__ void __launch_bounds__(256) k_rank_map(const uint8_t *__restrict__ in, uint64_t n,
                                                  int8_t *__restrict__ out, const int8_t *__restrict__ table,
                                                  unsigned long long *__restrict__ invalid)
{
    __shared__ uint32_t tab[64 * 32];
    for (int i = threadIdx.x; i < 64 * 32; i += blockDim.x) {
        const int w = i >> 5;
        tab[i] = (uint32_t)(uint8_t)table[4 * w] | ((uint32_t)(uint8_t)table[4 * w + 1] << 8) |
                 ((uint32_t)(uint8_t)table[4 * w + 2] << 16) | ((uint32_t)(uint8_t)table[4 * w + 3] << 24);
    }
    __syncthreads();
    const int lane = threadIdx.x & 31;
    const uint64_t tid = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x;
    const uint64_t nth = (uint64_t)gridDim.x * blockDim.x;
    unsigned bad = 0;                                   // ranks are 0..126: bit 7 marks "no rank"
    const bool vec = ((reinterpret_cast<uintptr_t>(in) | reinterpret_cast<uintptr_t>(out)) & 15) == 0;
    uint64_t done = 0;
    if (vec) {
        const uint64_t nv = n >> 4;
        for (uint64_t v0 = tid; v0 < nv; v0 += kUnroll * nth) {
            uint4 x[kUnroll];
#pragma unroll
            for (int u = 0; u < kUnroll; ++u) {
                const uint64_t v = v0 + u * nth;
                x[u] = v < nv ? __ldcs(reinterpret_cast<const uint4 *>(in) + v) : make_uint4(0, 0, 0, 0);
            }
#pragma unroll
            for (int u = 0; u < kUnroll; ++u) {
                const uint64_t v = v0 + u * nth;
                if (v >= nv) break;
                uint4 y;
                y.x = rank4(tab, lane, x[u].x);
                y.y = rank4(tab, lane, x[u].y);
                y.z = rank4(tab, lane, x[u].z);
                y.w = rank4(tab, lane, x[u].w);
                bad += __popc(y.x & 0x80808080u) + __popc(y.y & 0x80808080u) + __popc(y.z & 0x80808080u) +
                       __popc(y.w & 0x80808080u);
                __stcs(reinterpret_cast<uint4 *>(out) + v, y);
            }
        }
        done = nv << 4;
    }
    for (uint64_t i = done + tid; i < n; i += nth) {    // the tail, or everything when unaligned
        const uint32_t r = rank4(tab, lane, in[i]) & 0xffu;
        bad += r >> 7;
        out[i] = (int8_t)r;
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) bad += __shfl_xor_sync(0xffffffffu, bad, o);
    if (lane == 0 && bad) atomicAdd(invalid, (unsigned long long)bad);
}

// ---------------------------------------------------------------------------------------------
// 2-bit packing.  For the letters, ((b >> 1) ^ (b >> 2)) & 3 is A/a 0, C/c 1, G/g 2, T/t 3, so
// four bytes of a word are coded at once with no lookup; a byte is a DNA letter when b | 0x20 is
// one of a c g t.
// ---------------------------------------------------------------------------------------------
__device__ __forceinline__ uint32_t pack4(uint32_t w, unsigned &bad)
{
    const uint32_t x = ((w >> 1) ^ (w >> 2)) & 0x03030303u;          // codes at bits 0, 8, 16, 24
    // the lower-case letter each code stands for (one PRMT); a byte is valid when b | 0x20 is it
    const uint32_t sel = (x & 3u) | ((x >> 4) & 0x30u) | ((x >> 8) & 0x300u) | ((x >> 12) & 0x3000u);
    const uint32_t diff = (w | 0x20202020u) ^ __byte_perm(0x74676361u, 0u, sel);
    // bit 7 of a byte of z is set exactly when that byte of diff is zero (no carries between bytes)
    const uint32_t z = ~(((diff & 0x7f7f7f7fu) + 0x7f7f7f7fu) | diff | 0x7f7f7f7fu);
    bad += 4u - __popc(z);
    const uint32_t y = x | (x >> 6);                                   // codes at bits 0-3, 16-19
    return (y & 0xfu) | ((y >> 12) & 0xf0u);
}

__global__ void __launch_bounds__(256) k_pack_2bit(const uint8_t *__restrict__ in, uint64_t n,
                                                   uint32_t *__restrict__ words,
                                                   unsigned long long *__restrict__ invalid)
{
    const uint64_t tid = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x;
    const uint64_t nth = (uint64_t)gridDim.x * blockDim.x;
    const uint64_t nfull = n >> 4, nwords = (n + 15) >> 4;
    const bool vec = (reinterpret_cast<uintptr_t>(in) & 15) == 0;
    unsigned bad = 0;
    uint64_t first_slow = 0;
    if (vec) {
        for (uint64_t v0 = tid; v0 < nfull; v0 += kUnroll * nth) {
            uint4 x[kUnroll];
#pragma unroll
            for (int u = 0; u < kUnroll; ++u) {
                const uint64_t v = v0 + u * nth;
                x[u] = v < nfull ? __ldcs(reinterpret_cast<const uint4 *>(in) + v) : make_uint4(0, 0, 0, 0);
            }
#pragma unroll
            for (int u = 0; u < kUnroll; ++u) {
                const uint64_t v = v0 + u * nth;
                if (v >= nfull) break;
                words[v] = pack4(x[u].x, bad) | (pack4(x[u].y, bad) << 8) | (pack4(x[u].z, bad) << 16) |
                           (pack4(x[u].w, bad) << 24);
            }
        }
        first_slow = nfull;
    }
    for (uint64_t v = first_slow + tid; v < nwords; v += nth) {
        uint32_t w[4];
        {
            // unaligned input or the last partial word: byte loads; missing bytes act as 'A'
            // (code 0) and are not counted
            const uint64_t base = v << 4;
#pragma unroll
            for (int k = 0; k < 4; ++k) {
                uint32_t a = 0;
#pragma unroll
                for (int b = 0; b < 4; ++b) {
                    const uint64_t i = base + 4 * k + b;
                    a |= (uint32_t)(i < n ? in[i] : (uint8_t)'A') << (8 * b);
                }
                w[k] = a;
            }
        }
        const uint32_t out = pack4(w[0], bad) | (pack4(w[1], bad) << 8) | (pack4(w[2], bad) << 16) |
                             (pack4(w[3], bad) << 24);
        words[v] = out;
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) bad += __shfl_xor_sync(0xffffffffu, bad, o);
    if ((threadIdx.x & 31) == 0 && bad) atomicAdd(invalid, (unsigned long long)bad);
}

__device__ __forceinline__ uint32_t unpack4(uint32_t x)
{
    const uint32_t s = (x & 3u) | ((x & 0xcu) << 2) | ((x & 0x30u) << 4) | ((x & 0xc0u) << 6);
    return __byte_perm(0x54474341u, 0u, s);                         // bytes 'A' 'C' 'G' 'T'
}

// Bases [first_base, first_base + n) of the packed stream `words` -> letters out[0, n).
__global__ void __launch_bounds__(256) k_unpack_2bit(const uint32_t *__restrict__ words, uint64_t first_base,
                                                     uint64_t n, uint8_t *__restrict__ out)
{
    const uint64_t tid = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x;
    const uint64_t nth = (uint64_t)gridDim.x * blockDim.x;
    const uint32_t sh = (uint32_t)(first_base & 15) * 2;
    const uint64_t last_word = n ? (first_base + n - 1) >> 4 : 0;
    const bool vec = (reinterpret_cast<uintptr_t>(out) & 15) == 0;
    const uint64_t nt = (n + 15) >> 4;
    for (uint64_t t0 = tid; t0 < nt; t0 += kUnroll * nth) {
        uint32_t lo[kUnroll], hi[kUnroll];
#pragma unroll
        for (int u = 0; u < kUnroll; ++u) {
            const uint64_t t = t0 + u * nth;
            const uint64_t q = (first_base >> 4) + t;
            lo[u] = t < nt ? __ldg(words + q) : 0u;
            hi[u] = (t < nt && sh && q + 1 <= last_word) ? __ldg(words + q + 1) : 0u;
        }
#pragma unroll
        for (int u = 0; u < kUnroll; ++u) {
        const uint64_t t = t0 + u * nth;
        if (t >= nt) break;
        const uint32_t bits = sh ? __funnelshift_r(lo[u], hi[u], sh) : lo[u];
        uint4 y;
        y.x = unpack4(bits & 0xffu);
        y.y = unpack4((bits >> 8) & 0xffu);
        y.z = unpack4((bits >> 16) & 0xffu);
        y.w = unpack4(bits >> 24);
        const uint64_t o = t << 4;
        if (o + 16 <= n && vec) {
            __stcs(reinterpret_cast<uint4 *>(out + o), y);
        } else {
            const uint32_t v[4] = {y.x, y.y, y.z, y.w};
            for (int b = 0; b < 16 && o + b < n; ++b) out[o + b] = (uint8_t)(v[b >> 2] >> (8 * (b & 3)));
        }
        }
    }
}

static int stream_grid(int sm_count, uint64_t units)
{
    const uint64_t want = (units + 255) / 256;
    const uint64_t cap = (uint64_t)std::max(sm_count, 1) * 8;      // 8 blocks of 256 per SM
    return (int)std::max<uint64_t>(1, std::min(want, cap));
}

void rank_map_launch(const uint8_t *in, uint64_t n, int8_t *out, const int8_t *table, unsigned long long *invalid,
                     int sm_count, cudaStream_t st)
{
    k_rank_map<<<stream_grid(sm_count, (n + 15) / 16), 256, 0, st>>>(in, n, out, table, invalid);
}

void pack_2bit_launch(const uint8_t *in, uint64_t n, uint32_t *words, unsigned long long *invalid, int sm_count,
                      cudaStream_t st)
{
    k_pack_2bit<<<stream_grid(sm_count, (n + 15) / 16), 256, 0, st>>>(in, n, words, invalid);
}

void unpack_2bit_launch(const uint32_t *words, uint64_t first_base, uint64_t n, uint8_t *out, int sm_count,
                        cudaStream_t st)
{
    k_unpack_2bit<<<stream_grid(sm_count, (n + 15) / 16), 256, 0, st>>>(words, first_base, n, out);
}

}  // namespace pa

// ---------------------------------------------------------------------------------------------
// Host encoder: the same code and validity rule as k_pack_2bit, one byte at a time.
// ---------------------------------------------------------------------------------------------
pa_status pa_pack_2bit_host(const uint8_t *in, uint64_t n, uint32_t *out_words, uint64_t *n_invalid)
{
    if ((n && (!in || !out_words))) return PA_ERR_INVALID_ARGUMENT;
    uint64_t bad = 0;
    const uint64_t nwords = (n + 15) >> 4;
    for (uint64_t v = 0; v < nwords; ++v) {
        uint32_t w = 0;
        const uint64_t base = v << 4;
        const int cnt = (int)std::min<uint64_t>(16, n - base);
        for (int k = 0; k < cnt; ++k) {
            const uint8_t b = in[base + k];
            const uint8_t lower = b | 0x20;
            bad += !(lower == 'a' || lower == 'c' || lower == 'g' || lower == 't');
            w |= (uint32_t)(((b >> 1) ^ (b >> 2)) & 3) << (2 * k);
        }
        out_words[v] = w;
    }
    if (n_invalid) *n_invalid = bad;
    return PA_OK;
}

// ---------------------------------------------------------------------------------------------
// FASTA / FASTQ reader
// ---------------------------------------------------------------------------------------------
struct pa_seqfile {
    std::vector<uint8_t> seq, qual;
    std::vector<uint64_t> off{0};
    std::vector<uint64_t> name_off{0};
    std::string names;            // NUL-terminated names, back to back
    bool fastq = false;
};

namespace {

struct LineReader {
    const char *p, *end;
    uint64_t line = 0;
    // next line without its end ('\n', and a '\r' before it); false at the end of the text
    bool next(const char *&b, const char *&e)
    {
        if (p >= end) return false;
        b = p;
        const char *nl = static_cast<const char *>(std::memchr(p, '\n', (size_t)(end - p)));
        e = nl ? nl : end;
        p = nl ? nl + 1 : end;
        ++line;
        while (e > b && (e[-1] == '\r' || e[-1] == ' ' || e[-1] == '\t')) --e;
        return true;
    }
    bool peek_blank_or_end()
    {
        const char *q = p;
        while (q < end && (*q == ' ' || *q == '\t' || *q == '\r')) ++q;
        return q >= end || *q == '\n';
    }
};

pa_status seq_error(char *err, size_t len, uint64_t line, const char *why)
{
    if (err && len) std::snprintf(err, len, "line %llu: %s", (unsigned long long)line, why);
    return PA_ERR_INVALID_ARGUMENT;
}

void add_name(pa_seqfile &f, const char *b, const char *e)
{
    f.names.append(b, (size_t)(e - b));
    f.names.push_back('\0');
    f.name_off.push_back(f.names.size());
}

pa_status parse(const char *text, uint64_t len, pa_seqfile &f, char *err, size_t err_len)
{
    LineReader r{text, text + len};
    const char *b = nullptr, *e = nullptr;
    // the first non-blank line decides the format
    for (;;) {
        if (!r.next(b, e)) return PA_OK;                             // empty file: no records
        if (e > b) break;
    }
    if (*b != '>' && *b != '@') return seq_error(err, err_len, r.line, "expected '>' (FASTA) or '@' (FASTQ)");
    f.fastq = *b == '@';
    if (!f.fastq) {
        add_name(f, b + 1, e);
        while (r.next(b, e)) {
            if (e == b) continue;
            if (*b == '>') {
                f.off.push_back(f.seq.size());
                add_name(f, b + 1, e);
                continue;
            }
            for (const char *c = b; c < e; ++c)
                if (*c != ' ' && *c != '\t' && *c != '\r') f.seq.push_back((uint8_t)*c);
        }
        f.off.push_back(f.seq.size());
        return PA_OK;
    }
    for (;;) {
        // b..e is the '@' header line
        if (*b != '@') return seq_error(err, err_len, r.line, "expected '@' at the start of a FASTQ record");
        add_name(f, b + 1, e);
        const uint64_t start = f.seq.size();
        bool plus = false;
        while (r.next(b, e)) {
            if (e > b && *b == '+') { plus = true; break; }
            f.seq.insert(f.seq.end(), (const uint8_t *)b, (const uint8_t *)e);
        }
        if (!plus) return seq_error(err, err_len, r.line, "record without a '+' line");
        const uint64_t want = f.seq.size() - start;
        uint64_t got = 0;
        while (got < want) {
            if (!r.next(b, e)) return seq_error(err, err_len, r.line, "quality shorter than the sequence");
            f.qual.insert(f.qual.end(), (const uint8_t *)b, (const uint8_t *)e);
            got += (uint64_t)(e - b);
        }
        if (got != want) return seq_error(err, err_len, r.line, "quality longer than the sequence");
        f.off.push_back(f.seq.size());
        // an empty sequence has an empty quality line
        if (want == 0 && !r.peek_blank_or_end()) {
            const char *q = r.p;
            if (q < r.end && *q != '@') {
                r.next(b, e);
                if (e != b) return seq_error(err, err_len, r.line, "quality longer than the sequence");
            }
        }
        for (;;) {
            if (!r.next(b, e)) return PA_OK;
            if (e > b) break;
        }
    }
}

}  // namespace

pa_status pa_seqfile_parse(const char *text, uint64_t len, pa_seqfile **out, char *err, size_t err_len)
{
    if (!out || (len && !text)) return PA_ERR_INVALID_ARGUMENT;
    *out = nullptr;
    if (err && err_len) err[0] = '\0';
    pa_seqfile *f = new (std::nothrow) pa_seqfile;
    if (!f) return PA_ERR_OUT_OF_MEMORY;
    pa_status s;
    try {
        s = parse(text, len, *f, err, err_len);
    } catch (const std::bad_alloc &) {
        s = PA_ERR_OUT_OF_MEMORY;
    }
    if (s) {
        delete f;
        return s;
    }
    *out = f;
    return PA_OK;
}

pa_status pa_seqfile_read(const char *path, pa_seqfile **out, char *err, size_t err_len)
{
    if (!path || !out) return PA_ERR_INVALID_ARGUMENT;
    *out = nullptr;
    FILE *fp = std::fopen(path, "rb");
    if (!fp) {
        if (err && err_len) std::snprintf(err, err_len, "cannot open %s", path);
        return PA_ERR_INVALID_ARGUMENT;
    }
    std::vector<char> buf;
    char chunk[1 << 16];
    size_t got;
    try {
        while ((got = std::fread(chunk, 1, sizeof(chunk), fp)) > 0) buf.insert(buf.end(), chunk, chunk + got);
    } catch (const std::bad_alloc &) {
        std::fclose(fp);
        return PA_ERR_OUT_OF_MEMORY;
    }
    const bool failed = std::ferror(fp) != 0;
    std::fclose(fp);
    if (failed) {
        if (err && err_len) std::snprintf(err, err_len, "read error on %s", path);
        return PA_ERR_INVALID_ARGUMENT;
    }
    return pa_seqfile_parse(buf.data(), buf.size(), out, err, err_len);
}

uint64_t pa_seqfile_count(const pa_seqfile *f) { return f ? f->off.size() - 1 : 0; }
const uint8_t *pa_seqfile_sequences(const pa_seqfile *f) { return f ? f->seq.data() : nullptr; }
const uint64_t *pa_seqfile_offsets(const pa_seqfile *f) { return f ? f->off.data() : nullptr; }
const uint8_t *pa_seqfile_qualities(const pa_seqfile *f) { return f && f->fastq ? f->qual.data() : nullptr; }
const char *pa_seqfile_name(const pa_seqfile *f, uint64_t i)
{
    if (!f || i + 1 >= f->name_off.size()) return nullptr;
    return f->names.data() + f->name_off[i];
}
void pa_seqfile_free(pa_seqfile *f) { delete f; }
