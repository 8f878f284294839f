// readCSV (src/io.cpp:16-81) on the GPU: the file is streamed to the device
// through a small pinned ring (reader threads fill one bank of slots while
// the previous bank's copies run), then split and parsed there.
//
//   1. newline positions: per-64 KiB-chunk counts, a scan, and an ordered
//      write of each chunk's positions;
//   2. one thread per data row: the row's comma-separated pieces, with the
//      reference's getline behaviour (a field past the last piece repeats
//      the last piece; a row ending in ',' yields an empty field), and the
//      7 numeric fields through a device restatement of std::stod;
//   3. rows the device leaves undecided (hexadecimal, inf/nan, more than 19
//      significant digits, results out of the normal range, and conversions
//      within two units of a rounding boundary -- about 2^-70 of random
//      inputs) are parsed on the host with std::stod's own rules;
//   4. a scan over the valid rows numbers the bodies (the reference's ids)
//      and writes them, up to body_count, as the reference stops reading.
//
// Decimal to binary64: w * 10^q with w < 2^64 (at most 19 significant
// digits).  Exact operands take one rounding (w <= 2^53, |q| <= 22); exact
// dyadic values (5^-q divides w) convert the integer quotient; otherwise w
// times a 128-bit approximation of 5^q (bh_pow5_table.h) gives the leading
// 54 bits and the remainder of the product, whose error is below two units
// of the remainder; for 0 <= q <= 55 the table is exact and so is the
// decision.  This is the multiply-by-a-truncated-power scheme of Eisel and
// Lemire ("Number parsing at a gigabyte per second", 2021), restated.
#include "bh_internal.cuh"

#include <fcntl.h>
#include <sys/stat.h>
#include <unistd.h>

#include <algorithm>
#include <atomic>
#include <cerrno>
#include <cstdio>
#include <cstring>
#include <string>
#include <thread>
#include <vector>

#include "bh_pow5_table.h"

namespace {

constexpr int64_t kChunk = 1 << 16;  // bytes per newline-scan block
constexpr int kChunkThreads = 256;

__device__ const double kPow10[23] = {1e0,  1e1,  1e2,  1e3,  1e4,  1e5,  1e6,  1e7,  1e8,  1e9,  1e10, 1e11,
                                      1e12, 1e13, 1e14, 1e15, 1e16, 1e17, 1e18, 1e19, 1e20, 1e21, 1e22};

enum : uint8_t { kRowOk = 0, kRowBad = 1, kRowHost = 2 };

__device__ __forceinline__ bool is_space(char c) { return c == ' ' || (c >= '\t' && c <= '\r'); }

// RN(w 10^q) with the sign; 0 = done, kRowHost = undecided here.
__device__ int dec_to_double(uint64_t w, int q, bool neg, double* out)
{
    const uint64_t sgn = neg ? (1ull << 63) : 0ull;
    if (w == 0) {
        *out = __longlong_as_double((long long)sgn);
        return kRowOk;
    }
    if (q < kPow5Min || q > kPow5Max) return kRowHost;
    if (w <= (1ull << 53) && q >= -22 && q <= 22) {  // exact operands: one rounding
        const double x = (double)w;
        const double r = q >= 0 ? __dmul_rn(x, kPow10[q]) : __ddiv_rn(x, kPow10[-q]);
        *out = neg ? -r : r;
        return kRowOk;
    }
    if (q < 0 && q >= -27) {  // 5^-q < 2^63: an exact dyadic value when 5^-q divides w
        uint64_t p5 = 1;
        for (int k = 0; k < -q; ++k) p5 *= 5;
        if (w % p5 == 0) {
            const long long xb = __double_as_longlong(__ull2double_rn(w / p5));
            const int be = (int)((xb >> 52) & 0x7FF) + q;  // times 2^q
            if (be <= 0) return kRowHost;
            *out = __longlong_as_double((xb & ~(0x7FFll << 52)) | ((long long)be << 52) | (long long)sgn);
            return kRowOk;
        }
    }
    const int idx = q - kPow5Min;
    const uint64_t fh = kPow5Hi[idx], fl = kPow5Lo[idx];
    const int s = kPow5Shift[idx];
    const bool exact = q >= 0 && q <= kPow5ExactMax;
    const int lz = __clzll((long long)w);
    const uint64_t wn = w << lz;
    // Z = wn (fh 2^64 + fl); top = floor(Z / 2^64) (127 or 128 bits), low = Z mod 2^64
    const uint64_t a_lo = wn * fh, a_hi = __umul64hi(wn, fh);
    const uint64_t b_lo = wn * fl, b_hi = __umul64hi(wn, fl);
    const uint64_t t_lo = a_lo + b_hi;
    const uint64_t t_hi = a_hi + (t_lo < a_lo ? 1ull : 0ull);
    const int sh = (t_hi >> 63) ? 10 : 9;  // bits of t_hi below the 54 leading bits
    const uint64_t m54 = t_hi >> sh;
    const uint64_t r_hi = t_hi & ((1ull << sh) - 1), r_lo = t_lo;
    if (!exact) {
        const bool near_zero = r_hi == 0 && r_lo <= 1;
        const bool near_full = r_hi == (1ull << sh) - 1 && r_lo >= ~1ull;
        if (near_zero || near_full) return kRowHost;
    }
    uint64_t mant = m54 >> 1;
    bool up = false;
    if (m54 & 1) up = exact ? ((r_hi | r_lo | b_lo) != 0 || (mant & 1)) : true;
    mant += up ? 1 : 0;
    int E = (sh + 64) + 64 + s + q - lz + 1;  // value = mant 2^E
    if (mant == (1ull << 53)) {
        mant >>= 1;
        ++E;
    }
    const int be = E + 52 + 1023;
    if (be >= 2047 || be <= 0) return kRowHost;  // overflow (ERANGE) or subnormal: the host decides
    *out = __longlong_as_double((long long)(((uint64_t)be << 52) | (mant & ((1ull << 52) - 1)) | sgn));
    return kRowOk;
}

// std::stod over [s, e): kRowOk with *out, kRowBad (no conversion), kRowHost.
__device__ int parse_number(const char* s, const char* e, double* out)
{
    while (s < e && is_space(*s)) ++s;
    bool neg = false;
    if (s < e && (*s == '+' || *s == '-')) {
        neg = *s == '-';
        ++s;
    }
    if (s >= e) return kRowBad;
    const char c0 = *s;
    if (!((c0 >= '0' && c0 <= '9') || c0 == '.')) {
        const char l = (char)(c0 | 0x20);
        return (l == 'i' || l == 'n') ? kRowHost : kRowBad;  // inf, infinity, nan
    }
    if (c0 == '0' && s + 1 < e && (s[1] | 0x20) == 'x') return kRowHost;  // hexadecimal
    uint64_t w = 0;
    int nd = 0, q = 0;
    bool any = false, trunc = false;
    while (s < e && *s >= '0' && *s <= '9') {
        any = true;
        if (!(w == 0 && *s == '0')) {
            if (nd < 19) {
                w = w * 10 + (uint64_t)(*s - '0');
                ++nd;
            } else {
                ++q;
                trunc |= *s != '0';
            }
        }
        ++s;
    }
    if (s < e && *s == '.') {
        ++s;
        while (s < e && *s >= '0' && *s <= '9') {
            any = true;
            if (w == 0 && *s == '0') {
                --q;
            } else if (nd < 19) {
                w = w * 10 + (uint64_t)(*s - '0');
                ++nd;
                --q;
            } else {
                trunc |= *s != '0';
            }
            ++s;
        }
    }
    if (!any) return kRowBad;
    if (s < e && (*s | 0x20) == 'e') {
        const char* t = s + 1;
        bool en = false;
        if (t < e && (*t == '+' || *t == '-')) {
            en = *t == '-';
            ++t;
        }
        if (t < e && *t >= '0' && *t <= '9') {
            int x = 0;
            while (t < e && *t >= '0' && *t <= '9') {
                if (x < 100000) x = x * 10 + (*t - '0');
                ++t;
            }
            q += en ? -x : x;
        }
    }
    if (trunc) return kRowHost;
    return dec_to_double(w, q, neg, out);
}

// 16 bytes per thread per round (one 128-bit load, coalesced): 4,096 bytes a
// round, 16 rounds a chunk.  Chunk starts are multiples of 64 KiB in a
// cudaMalloc buffer, so every full 16-byte group is 16-byte aligned; the
// file's last partial group is read byte by byte.
constexpr int kGroup = 16;
constexpr int64_t kRound = (int64_t)kGroup * kChunkThreads;

// Bytes i0 .. i0 + 15 (those below b) as four words, and a per-byte mask of
// newlines in each (0xFF where the byte is '\n', via the SIMD byte compare).
__device__ __forceinline__ void newline_masks(const char* __restrict__ buf, int64_t i0, int64_t b,
                                              unsigned m[4])
{
    unsigned v[4];
    if (i0 + kGroup <= b) {
        const uint4 q = __ldg(reinterpret_cast<const uint4*>(buf + i0));
        v[0] = q.x; v[1] = q.y; v[2] = q.z; v[3] = q.w;
    } else {
        for (int k = 0; k < 4; ++k) {
            unsigned w = 0;
            for (int j = 0; j < 4; ++j) {
                const int64_t i = i0 + 4 * k + j;
                const unsigned c = i < b ? (unsigned)(unsigned char)buf[i] : 0u;
                w |= c << (8 * j);
            }
            v[k] = w;
        }
    }
    for (int k = 0; k < 4; ++k) m[k] = __vcmpeq4(v[k], 0x0A0A0A0Au);
}

__device__ __forceinline__ int mask_count(const unsigned m[4])
{
    return (__popc(m[0]) + __popc(m[1]) + __popc(m[2]) + __popc(m[3])) >> 3;
}

__global__ void __launch_bounds__(kChunkThreads) nl_count_kernel(const char* __restrict__ buf, int64_t size,
                                                                 int32_t* __restrict__ cnt)
{
    const int64_t a = (int64_t)blockIdx.x * kChunk, b = min(a + kChunk, size);
    int c = 0;
    for (int64_t i0 = a + kGroup * (int64_t)threadIdx.x; i0 < b; i0 += kRound) {
        unsigned m[4];
        newline_masks(buf, i0, b, m);
        c += mask_count(m);
    }
    c = __reduce_add_sync(0xffffffffu, c);
    __shared__ int ws[kChunkThreads / 32];
    if ((threadIdx.x & 31) == 0) ws[threadIdx.x >> 5] = c;
    __syncthreads();
    if (threadIdx.x == 0) {
        int t = 0;
        for (int k = 0; k < kChunkThreads / 32; ++k) t += ws[k];
        cnt[blockIdx.x] = t;
    }
}

// The same rounds as nl_count_kernel: a block-wide exclusive scan of the
// per-thread counts places each round's positions after the previous
// round's, in file order.
__global__ void __launch_bounds__(kChunkThreads) nl_write_kernel(const char* __restrict__ buf, int64_t size,
                                                                 const int32_t* __restrict__ off,
                                                                 int64_t* __restrict__ nl_pos)
{
    __shared__ int warp_tot[kChunkThreads / 32];
    __shared__ int round_tot;
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    const int64_t a = (int64_t)blockIdx.x * kChunk, b = min(a + kChunk, size);
    int64_t o = off[blockIdx.x];
    for (int64_t r = a; r < b; r += kRound) {  // the same trip count in every thread
        const int64_t i0 = r + kGroup * (int64_t)threadIdx.x;
        unsigned m[4] = {0u, 0u, 0u, 0u};
        if (i0 < b) newline_masks(buf, i0, b, m);
        const int mine = mask_count(m);
        int incl = mine;
#pragma unroll
        for (int d = 1; d < 32; d <<= 1) {
            const int t = __shfl_up_sync(0xffffffffu, incl, d);
            if (lane >= d) incl += t;
        }
        if (lane == 31) warp_tot[w] = incl;
        __syncthreads();
        if (threadIdx.x == 0) {
            int run = 0;
            for (int k = 0; k < kChunkThreads / 32; ++k) {
                const int t = warp_tot[k];
                warp_tot[k] = run;
                run += t;
            }
            round_tot = run;
        }
        __syncthreads();
        int64_t p = o + warp_tot[w] + incl - mine;
        for (int k = 0; k < 4; ++k) {
            unsigned mk = m[k];
            while (mk) {
                const int byte = (__ffs(mk) - 1) >> 3;
                nl_pos[p++] = i0 + 4 * k + byte;
                mk &= ~(0xFFu << (8 * byte));
            }
        }
        o += round_tot;
        __syncthreads();
    }
}

// Data row d is line d + 1 (line 0 is the header).
__device__ __forceinline__ void row_bounds(int64_t d, const int64_t* nl_pos, int64_t nl, int64_t size, int64_t* a,
                                           int64_t* b)
{
    const int64_t line = d + 1;
    *a = nl_pos[line - 1] + 1;
    *b = line < nl ? nl_pos[line] : size;
}

__global__ void row_parse_kernel(const char* __restrict__ buf, int64_t size, const int64_t* __restrict__ nl_pos,
                                 int64_t nl, int64_t rows, double* __restrict__ vals, uint8_t* __restrict__ status)
{
    for (int64_t d = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; d < rows; d += (int64_t)gridDim.x * blockDim.x) {
        int64_t a, b;
        row_bounds(d, nl_pos, nl, size, &a, &b);
        // pieces 3..9 by commas; a field past the last piece repeats it
        int64_t ps[10], pe[10];
        int k = 0;
        int64_t st = a;
        for (int64_t i = a; i < b && k < 10; ++i) {
            if (buf[i] == ',') {
                ps[k] = st;
                pe[k] = i;
                ++k;
                st = i + 1;
            }
        }
        if (k < 10) {
            ps[k] = st;
            pe[k] = b;
            ++k;
        }
        uint8_t res = kRowOk;
        for (int f = 0; f < 7; ++f) {
            const int p = min(3 + f, k - 1);
            double v = 0.0;
            const int r = parse_number(buf + ps[p], buf + pe[p], &v);
            if (r != kRowOk) {
                res = (uint8_t)r;
                break;  // the reference stops at the first field that throws
            }
            vals[(int64_t)f * rows + d] = v;
        }
        status[d] = res;
    }
}

__global__ void row_fix_kernel(int nfix, const int64_t* __restrict__ fix_row, const uint8_t* __restrict__ fix_status,
                               const double* __restrict__ fix_vals, int64_t rows, double* __restrict__ vals,
                               uint8_t* __restrict__ status)
{
    const int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= nfix) return;
    const int64_t d = fix_row[k];
    status[d] = fix_status[k];
    for (int f = 0; f < 7; ++f) vals[(int64_t)f * rows + d] = fix_vals[7 * k + f];
}

__global__ void row_flag_kernel(int64_t rows, const uint8_t* __restrict__ status, int32_t* __restrict__ flag)
{
    for (int64_t d = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; d < rows; d += (int64_t)gridDim.x * blockDim.x)
        flag[d] = status[d] == kRowOk ? 1 : 0;
}

// Body idx (the reference's id) for valid row d, up to n bodies: SoA out.
__global__ void row_emit_kernel(int64_t rows, int64_t n, const uint8_t* __restrict__ status,
                                const int32_t* __restrict__ idx, const double* __restrict__ vals,
                                double* __restrict__ m, double* __restrict__ x, double* __restrict__ y,
                                double* __restrict__ z, double* __restrict__ vx, double* __restrict__ vy,
                                double* __restrict__ vz, uint64_t* __restrict__ id)
{
    for (int64_t d = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; d < rows; d += (int64_t)gridDim.x * blockDim.x) {
        if (status[d] != kRowOk) continue;
        const int64_t i = idx[d];
        if (i >= n) continue;
        m[i] = vals[d];
        x[i] = vals[rows + d];
        y[i] = vals[2 * rows + d];
        z[i] = vals[3 * rows + d];
        vx[i] = vals[4 * rows + d];
        vy[i] = vals[5 * rows + d];
        vz[i] = vals[6 * rows + d];
        id[i] = (uint64_t)i;
    }
}

struct DevBuf {
    void* p = nullptr;
    ~DevBuf()
    {
        if (p) cudaFree(p);
    }
    template <class T>
    T* as()
    {
        return static_cast<T*>(p);
    }
};

struct HostBuf {
    char* p = nullptr;
    ~HostBuf()
    {
        if (p) cudaFreeHost(p);
    }
};

struct FileFd {
    int fd = -1;
    ~FileFd()
    {
        if (fd >= 0) ::close(fd);
    }
};

struct Events {
    cudaEvent_t e[2] = {nullptr, nullptr};
    ~Events()
    {
        for (auto x : e)
            if (x) cudaEventDestroy(x);
    }
};

// Bytes [off, off + len) of the file, retrying short reads.
bool read_at(int fd, char* dst, int64_t off, int64_t len)
{
    while (len > 0) {
        const ssize_t r = ::pread(fd, dst, (size_t)len, (off_t)off);
        if (r < 0 && errno == EINTR) continue;
        if (r <= 0) return false;
        dst += r;
        off += r;
        len -= r;
    }
    return true;
}

bool text_at(int fd, int64_t a, int64_t b, std::string& t)
{
    t.assign((size_t)std::max<int64_t>(b - a, 0), '\0');
    return t.empty() || read_at(fd, &t[0], a, (int64_t)t.size());
}

constexpr int64_t kStage = 4 << 20;  // bytes per slot of the pinned ring
constexpr int kReaders = 4;          // slots per bank, one reader thread each

// The whole file to dst on the device, in order on stream st.  Two banks of
// kReaders slots: a bank's slots are read in parallel (one thread each, the
// caller's thread taking the first), then copied asynchronously; the bank is
// reused once its copies have completed (an event per bank).
int stream_file(int fd, int64_t size, char* dst, cudaStream_t st, const char* fn)
{
    const int64_t slots = 2 * kReaders;
    const int64_t ring = std::min<int64_t>(size, slots * kStage);
    HostBuf hb;
    if (cudaMallocHost(reinterpret_cast<void**>(&hb.p), (size_t)ring) != cudaSuccess) {
        cudaGetLastError();
        return bh_fail(BH_ERR_OUT_OF_MEMORY, std::string(fn) + ": pinned staging buffer");
    }
    Events ev;
    for (auto& x : ev.e) BH_CUDA_TRY(cudaEventCreateWithFlags(&x, cudaEventDisableTiming));
    const int64_t nchunks = (size + kStage - 1) / kStage;
    for (int64_t c0 = 0, round = 0; c0 < nchunks; c0 += kReaders, ++round) {
        const int bank = (int)(round & 1);
        if (round >= 2) BH_CUDA_TRY(cudaEventSynchronize(ev.e[bank]));
        const int k = (int)std::min<int64_t>(kReaders, nchunks - c0);
        std::atomic<bool> ok{true};
        auto slot = [&](int j) { return hb.p + (int64_t)(bank * kReaders + j) * kStage; };
        auto work = [&](int j) {
            const int64_t off = (c0 + j) * kStage;
            if (!read_at(fd, slot(j), off, std::min(kStage, size - off))) ok = false;
        };
        std::vector<std::thread> th;
        int spawned = 1;
        try {
            for (; spawned < k; ++spawned) th.emplace_back(work, spawned);
        } catch (...) {  // no thread to spare: the caller reads the rest
        }
        work(0);
        for (int j = spawned; j < k; ++j) work(j);
        for (auto& t : th) t.join();
        if (!ok) return bh_fail(BH_ERR_IO, std::string(fn) + ": short read");
        for (int j = 0; j < k; ++j) {
            const int64_t off = (c0 + j) * kStage;
            BH_CUDA_TRY(cudaMemcpyAsync(dst + off, slot(j), (size_t)std::min(kStage, size - off),
                                        cudaMemcpyHostToDevice, st));
        }
        BH_CUDA_TRY(cudaEventRecord(ev.e[bank], st));
    }
    BH_CUDA_TRY(cudaStreamSynchronize(st));  // the ring is freed on return
    return BH_OK;
}

struct Out7 {
    double *m, *x, *y, *z, *vx, *vy, *vz;
    uint64_t* id;
};

// The 8 arrays of n bodies in one device block (mass, x, y, z, vx, vy, vz,
// then the ids).
Out7 out7_of(double* b, int64_t n)
{
    return Out7{b, b + n, b + 2 * n, b + 3 * n, b + 4 * n, b + 5 * n, b + 6 * n, reinterpret_cast<uint64_t*>(b + 7 * n)};
}

// Parses `path` on ctx's device.  With `out` (room for `cap` bodies) the
// bodies are written there; otherwise, with `own`, into a block of exactly
// the body count allocated there (out7_of layout); *n_out is the body count
// either way.
int csv_parse(bh_context* ctx, const char* path, int64_t body_count, const Out7* out, int64_t cap, int64_t* n_out,
              const char* fn, DevBuf* own = nullptr)
{
    *n_out = 0;
    FileFd file;
    file.fd = ::open(path, O_RDONLY);
    if (file.fd < 0) return bh_fail(BH_ERR_IO, std::string(fn) + ": cannot open " + path);
    struct stat sb;
    if (::fstat(file.fd, &sb) != 0 || !S_ISREG(sb.st_mode))
        return bh_fail(BH_ERR_IO, std::string(fn) + ": cannot size " + path);
    const int64_t size = (int64_t)sb.st_size;
    if (size == 0) return BH_OK;
    char last = 0;
    if (!read_at(file.fd, &last, size - 1, 1)) return bh_fail(BH_ERR_IO, std::string(fn) + ": short read of " + path);

    cudaStream_t st = ctx->stream;
    const int64_t nch = (size + kChunk - 1) / kChunk;
    DevBuf dbuf, dcnt, dsmall;
    BH_CUDA_TRY(cudaMalloc(&dbuf.p, (size_t)size));
    BH_CUDA_TRY(cudaMalloc(&dcnt.p, sizeof(int32_t) * (size_t)(nch + bh::scan_tmp_ints(nch))));
    BH_CUDA_TRY(cudaMalloc(&dsmall.p, 64 * sizeof(int32_t)));
    int32_t* cnt = dcnt.as<int32_t>();
    int32_t* tmp = cnt + nch;
    int32_t* small = dsmall.as<int32_t>();
    int rc = stream_file(file.fd, size, dbuf.as<char>(), st, fn);
    if (rc) return rc;
    nl_count_kernel<<<(unsigned)nch, kChunkThreads, 0, st>>>(dbuf.as<char>(), size, cnt);
    BH_LAUNCH_CHECK(ctx);
    rc = bh::device_exclusive_scan_tmp(ctx, cnt, cnt, nch, nullptr, small, tmp);
    if (rc) return rc;
    BH_CUDA_TRY(cudaMemcpyAsync(ctx->h_small, small, sizeof(int32_t), cudaMemcpyDeviceToHost, st));
    BH_CUDA_TRY(cudaStreamSynchronize(st));
    int32_t nl32 = 0;
    std::memcpy(&nl32, ctx->h_small, sizeof(int32_t));
    const int64_t nl = nl32;
    const int64_t lines = nl + (last != '\n' ? 1 : 0);
    const int64_t rows = lines - 1;  // line 0 is the header
    if (rows <= 0) return BH_OK;
    if (rows >= (int64_t)INT32_MAX) return bh_fail(BH_ERR_INVALID_ARGUMENT, std::string(fn) + ": too many rows");

    DevBuf dnl, dvals, dstat, dflag;
    BH_CUDA_TRY(cudaMalloc(&dnl.p, sizeof(int64_t) * (size_t)std::max<int64_t>(nl, 1)));
    BH_CUDA_TRY(cudaMalloc(&dvals.p, sizeof(double) * 7 * (size_t)rows));
    BH_CUDA_TRY(cudaMalloc(&dstat.p, (size_t)rows));
    BH_CUDA_TRY(cudaMalloc(&dflag.p, sizeof(int32_t) * (size_t)(rows + bh::scan_tmp_ints(rows))));
    int64_t* nl_pos = dnl.as<int64_t>();
    double* vals = dvals.as<double>();
    uint8_t* status = dstat.as<uint8_t>();
    nl_write_kernel<<<(unsigned)nch, kChunkThreads, 0, st>>>(dbuf.as<char>(), size, cnt, nl_pos);
    BH_LAUNCH_CHECK(ctx);
    const int grid = (int)std::min<int64_t>((rows + 127) / 128, 64 * (int64_t)bh::num_sms());
    row_parse_kernel<<<grid, 128, 0, st>>>(dbuf.as<char>(), size, nl_pos, nl, rows, vals, status);
    BH_LAUNCH_CHECK(ctx);

    // Rows the device did not decide, and the warnings, on the host.
    std::vector<uint8_t> hst((size_t)rows);
    BH_CUDA_TRY(cudaMemcpyAsync(hst.data(), status, (size_t)rows, cudaMemcpyDeviceToHost, st));
    BH_CUDA_TRY(cudaStreamSynchronize(st));
    std::vector<int64_t> odd;  // rows not plainly valid
    for (int64_t d = 0; d < rows; ++d)
        if (hst[(size_t)d] != kRowOk) odd.push_back(d);
    std::vector<std::pair<int64_t, std::string>> bad_rows;
    if (!odd.empty()) {
        std::vector<int64_t> hnl((size_t)nl);
        BH_CUDA_TRY(cudaMemcpy(hnl.data(), nl_pos, sizeof(int64_t) * (size_t)nl, cudaMemcpyDeviceToHost));
        std::vector<int64_t> fix_row;
        std::vector<uint8_t> fix_status;
        std::vector<double> fix_vals;
        for (int64_t d : odd) {
            const int64_t a = hnl[(size_t)d] + 1, b = d + 1 < nl ? hnl[(size_t)(d + 1)] : size;
            std::string text;
            if (!text_at(file.fd, a, b, text)) return bh_fail(BH_ERR_IO, std::string(fn) + ": short read of " + path);
            if (hst[(size_t)d] == kRowHost) {
                double v[7] = {0, 0, 0, 0, 0, 0, 0};
                const bool ok = bh_parse_csv_row(text, v);
                hst[(size_t)d] = ok ? kRowOk : kRowBad;
                fix_row.push_back(d);
                fix_status.push_back(hst[(size_t)d]);
                fix_vals.insert(fix_vals.end(), v, v + 7);
            }
            if (hst[(size_t)d] == kRowBad) bad_rows.emplace_back(d, text);
        }
        if (!fix_row.empty()) {
            const int nfix = (int)fix_row.size();
            DevBuf dfix;
            BH_CUDA_TRY(cudaMalloc(&dfix.p, (sizeof(int64_t) + 1 + 7 * sizeof(double)) * (size_t)nfix + 64));
            int64_t* d_row = dfix.as<int64_t>();
            double* d_vals = reinterpret_cast<double*>(d_row + nfix);
            uint8_t* d_st = reinterpret_cast<uint8_t*>(d_vals + 7 * (size_t)nfix);
            BH_CUDA_TRY(cudaMemcpyAsync(d_row, fix_row.data(), sizeof(int64_t) * nfix, cudaMemcpyHostToDevice, st));
            BH_CUDA_TRY(cudaMemcpyAsync(d_vals, fix_vals.data(), sizeof(double) * 7 * nfix, cudaMemcpyHostToDevice, st));
            BH_CUDA_TRY(cudaMemcpyAsync(d_st, fix_status.data(), (size_t)nfix, cudaMemcpyHostToDevice, st));
            row_fix_kernel<<<(nfix + 255) / 256, 256, 0, st>>>(nfix, d_row, d_st, d_vals, rows, vals, status);
            BH_LAUNCH_CHECK(ctx);
            BH_CUDA_TRY(cudaStreamSynchronize(st));
        }
    }

    // Number the valid rows; the reference stops once body_count are read.
    int32_t* flag = dflag.as<int32_t>();
    row_flag_kernel<<<grid, 128, 0, st>>>(rows, status, flag);
    BH_LAUNCH_CHECK(ctx);
    if ((rc = bh::device_exclusive_scan_tmp(ctx, flag, flag, rows, nullptr, small + 1, flag + rows))) return rc;
    BH_CUDA_TRY(cudaMemcpyAsync(ctx->h_small, small + 1, sizeof(int32_t), cudaMemcpyDeviceToHost, st));
    BH_CUDA_TRY(cudaStreamSynchronize(st));
    int32_t valid = 0;
    std::memcpy(&valid, ctx->h_small, sizeof(int32_t));
    const int64_t n = body_count > 0 ? std::min<int64_t>(valid, body_count) : valid;
    // warnings for the rows the reference reads: those before the n-th valid row
    int64_t seen = 0, bi = 0;
    for (int64_t d = 0; d < rows && (body_count <= 0 || seen < body_count); ++d) {
        if (hst[(size_t)d] == kRowOk) {
            ++seen;
        } else if (hst[(size_t)d] == kRowBad) {
            while (bi < (int64_t)bad_rows.size() && bad_rows[(size_t)bi].first < d) ++bi;
            if (bi < (int64_t)bad_rows.size() && bad_rows[(size_t)bi].first == d)
                std::fprintf(stderr, "Warning: Could not parse line, skipping: \"%s\"\n",
                             bad_rows[(size_t)bi].second.c_str());
        }
    }
    *n_out = n;
    Out7 mine;
    if (!out && own && n > 0) {
        BH_CUDA_TRY(cudaMalloc(&own->p, sizeof(double) * 8 * (size_t)n));
        mine = out7_of(own->as<double>(), n);
        out = &mine;
        cap = n;
    }
    if (!out) return BH_OK;
    if (n > cap) return bh_fail(BH_ERR_CAPACITY, std::string(fn) + ": more bodies than the output holds");
    row_emit_kernel<<<grid, 128, 0, st>>>(rows, n, status, flag, vals, out->m, out->x, out->y, out->z, out->vx,
                                          out->vy, out->vz, out->id);
    BH_LAUNCH_CHECK(ctx);
    BH_CUDA_TRY(cudaStreamSynchronize(st));
    return BH_OK;
}

}  // namespace

extern "C" int bh_read_csv_gpu(const char* path, int64_t body_count, int64_t* n_out, uint64_t* ids, double* mass,
                               double* pos, double* vel)
{
    if (!path || !n_out) return bh_fail(BH_ERR_INVALID_ARGUMENT, "bh_read_csv_gpu: null path or n_out");
    const bool fill = pos != nullptr;
    if (fill && (!ids || !mass || !vel))
        return bh_fail(BH_ERR_INVALID_ARGUMENT, "bh_read_csv_gpu: missing output arrays");
    int dev = 0;
    BH_CUDA_TRY(cudaGetDevice(&dev));
    bh_context* ctx = nullptr;
    int rc = bh_context_create(1, dev, &ctx);
    if (rc) return rc;
    struct Guard {
        bh_context* c;
        ~Guard() { bh_context_destroy(c); }
    } guard{ctx};
    if (!fill) return csv_parse(ctx, path, body_count, nullptr, 0, n_out, "bh_read_csv_gpu");
    // One parse into a device block of the body count, then to the caller's
    // arrays (room for the count of the sizing call on the same file).
    int64_t n = 0;
    DevBuf d;
    if ((rc = csv_parse(ctx, path, body_count, nullptr, 0, &n, "bh_read_csv_gpu", &d))) return rc;
    *n_out = n;
    if (n == 0) return BH_OK;
    const double* b = d.as<double>();
    std::vector<double> h(8 * (size_t)n);
    BH_CUDA_TRY(cudaMemcpy(h.data(), b, sizeof(double) * 8 * (size_t)n, cudaMemcpyDeviceToHost));
    for (int64_t i = 0; i < n; ++i) {
        mass[i] = h[(size_t)i];
        for (int a = 0; a < 3; ++a) {
            pos[3 * i + a] = h[(size_t)((1 + a) * n + i)];
            vel[3 * i + a] = h[(size_t)((4 + a) * n + i)];
        }
    }
    std::memcpy(ids, h.data() + 7 * (size_t)n, sizeof(uint64_t) * (size_t)n);
    return BH_OK;
}

extern "C" int bh_load_csv(bh_context* ctx, const char* path, int64_t body_count, int64_t* n_out)
{
    if (!ctx || !path || !n_out) return bh_fail(BH_ERR_INVALID_ARGUMENT, "bh_load_csv: bad arguments");
    BH_CUDA_TRY(cudaSetDevice(ctx->device));
    const Out7 o{ctx->m, ctx->px, ctx->py, ctx->pz, ctx->vx, ctx->vy, ctx->vz, ctx->id};
    int64_t n = 0;
    const int rc = csv_parse(ctx, path, body_count, &o, ctx->cap, &n, "bh_load_csv");
    *n_out = n;
    if (rc) return rc;
    ctx->n = n;
    ctx->t = 0.0;
    ctx->tree_valid = ctx->keys_valid = ctx->bbox_valid = ctx->sorted_valid = false;
    if (n > 0) {
        BH_CUDA_TRY(cudaMemsetAsync(ctx->ax, 0, sizeof(double) * n, ctx->stream));
        BH_CUDA_TRY(cudaMemsetAsync(ctx->ay, 0, sizeof(double) * n, ctx->stream));
        BH_CUDA_TRY(cudaMemsetAsync(ctx->az, 0, sizeof(double) * n, ctx->stream));
        BH_CUDA_TRY(cudaStreamSynchronize(ctx->stream));
    }
    return BH_OK;
}
