// frame.cu -- particle frames in the reference's text format, formatted on the device.
//
// SerializerSaveSphDataSet3 (src/third/serializer.cpp:880-923) appends a block
//   FluidBegin / "Type" particles / "Count" n / "Format" <flags> / "Spacing" h0 /
//   DataBegin / one line per particle / DataEnd / FluidEnd
// where each particle line is two tabs, the selected fields as %g numbers separated by
// spaces (position, velocity, density, mass; PushParticleSetToFile, :824-878) and a newline.
// Here one thread formats one particle's line (caller order) into a fixed-size slot with
// the exact %g of gfmt.h, an exclusive scan of the line lengths gives each line's offset,
// and a second pass packs the lines into one contiguous buffer: the host receives only the
// bytes of the frame.
#include "bbg_kernels.h"
#include "frame.h"
#include "gfmt.h"

#include <cmath>
#include <cstring>

namespace bbg {

static inline int blocks_for(long long n, int t) { return (int)((n + t - 1) / t); }

__device__ __forceinline__ void put3(char *line, int &len, float4 v, bool space) {
    if (space) line[len++] = ' ';
    len += gfmt::format_g(v.x, line + len);
    line[len++] = ' ';
    len += gfmt::format_g(v.y, line + len);
    line[len++] = ' ';
    len += gfmt::format_g(v.z, line + len);
}

__global__ void k_frame_lines(int n, int flags, const float4 *__restrict__ pos, const float4 *__restrict__ vel,
                              const float *__restrict__ rho, const int *__restrict__ slot, float mass,
                              char *__restrict__ lines, unsigned *__restrict__ lens) {
    const int id = blockIdx.x * blockDim.x + threadIdx.x;
    if (id >= n) return;
    const int s = slot[id];
    char *line = lines + (size_t)id * kFrameLineCap;
    int len = 0;
    line[len++] = '\t';
    line[len++] = '\t';
    bool space = false;
    if (flags & kFramePosition) {
        put3(line, len, pos[s], space);
        space = true;
    }
    if (flags & kFrameVelocity) {
        put3(line, len, vel[s], space);
        space = true;
    }
    if (flags & kFrameDensity) {
        if (space) line[len++] = ' ';
        len += gfmt::format_g(rho[s], line + len);
        space = true;
    }
    if (flags & kFrameMass) {
        if (space) line[len++] = ' ';
        len += gfmt::format_g(mass, line + len);
    }
    line[len++] = '\n';
    lens[id] = (unsigned)len;
}

__global__ void k_frame_pack(int n, const char *__restrict__ lines, const unsigned *__restrict__ offset,
                             const unsigned *__restrict__ lens, char *__restrict__ out) {
    const int id = blockIdx.x * blockDim.x + threadIdx.x;
    if (id >= n) return;
    const char *src = lines + (size_t)id * kFrameLineCap;
    char *dst = out + offset[id];
    const unsigned len = lens[id];
    for (unsigned k = 0; k < len; k++) dst[k] = src[k];
}

void launch_frame_lines(int n, int flags, const float4 *pos, const float4 *vel, const float *rho,
                        const int *slot, float mass, FrameBufs &F, cudaStream_t s) {
    k_frame_lines<<<blocks_for(n, 128), 128, 0, s>>>(n, flags, pos, vel, rho, slot, mass, F.lines, F.lens);
    // the scan consumes its input: keep the lengths for the packing pass
    cudaMemcpyAsync(F.scan_in, F.lens, sizeof(unsigned) * (size_t)n, cudaMemcpyDeviceToDevice, s);
    launch_cell_scan(F.scan_in, (unsigned)n, F.partials, F.offset, s);
    k_frame_pack<<<blocks_for(n, 128), 128, 0, s>>>(n, F.lines, F.offset, F.lens, F.out);
}

// ----------------------------------------------------------------------------
// reading: SerializerLoadParticles3 (src/third/serializer.cpp:450-560) on the device
// ----------------------------------------------------------------------------
// GetLine (src/third/obj_loader.cpp:253-268) ends a line at "\n", "\r\n" or "\r": byte i
// starts a line if i == 0, the byte before is '\n', or it is '\r' not followed by '\n'.
__device__ __forceinline__ bool starts_line(const char *t, size_t i) {
    if (i == 0) return true;
    const char p = t[i - 1];
    return p == '\n' || (p == '\r' && t[i] != '\n');
}

__global__ void k_line_count(const char *__restrict__ t, size_t bytes, unsigned *__restrict__ chunk) {
    const size_t c = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    const size_t lo = c * kLineChunk;
    if (lo >= bytes) return;
    const size_t hi = lo + kLineChunk < bytes ? lo + kLineChunk : bytes;
    unsigned k = 0;
    for (size_t i = lo; i < hi; i++) k += starts_line(t, i) ? 1u : 0u;
    chunk[c] = k;
}

__global__ void k_line_write(const char *__restrict__ t, size_t bytes, const unsigned *__restrict__ chunk_start,
                             unsigned *__restrict__ line) {
    const size_t c = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    const size_t lo = c * kLineChunk;
    if (lo >= bytes) return;
    const size_t hi = lo + kLineChunk < bytes ? lo + kLineChunk : bytes;
    unsigned k = chunk_start[c];
    for (size_t i = lo; i < hi; i++)
        if (starts_line(t, i)) line[k++] = (unsigned)i;
}

__device__ __forceinline__ bool is_digit(char c) { return (unsigned)(c - '0') < 10u; }

// x * 2^e for the e the reader can meet with a finite x (|e| <= 1023); like ldexp, one
// rounding at most (subnormal results), inf on overflow.
__device__ __forceinline__ double scale2(double x, int e) {
    if (e < -1022 || e > 1023) return x;   // x is 0, inf or nan there: pow(5, e) over/underflowed
    return __dmul_rn(x, __longlong_as_double((long long)(e + 1023) << 52));
}

// ParseFloat's number reader (src/third/obj_loader.cpp:56-168) in the same double
// operations, unfused: mantissa = mantissa * 10 + digit, fraction digits weighted by
// 0.1 .. 1e-7 and pow(10, -r) beyond, exponent applied as ldexp(m * pow(5, e), e) with
// the pow values of the host's libm; a malformed token reads as 0.
__device__ double parse_number(const char *s, const char *end, const double *__restrict__ pow5,
                               const double *__restrict__ pow10) {
    if (s >= end) return 0.0;
    const char *c = s;
    double mantissa = 0.0;
    int exponent = 0, read = 0;
    bool neg = false, eneg = false;
    if (*c == '+' || *c == '-') {
        neg = *c == '-';
        c++;
    } else if (!is_digit(*c)) {
        return 0.0;
    }
    while (c != end && is_digit(*c)) {
        mantissa = __dadd_rn(__dmul_rn(mantissa, 10.0), (double)(*c - '0'));
        c++;
        read++;
    }
    if (read == 0) return 0.0;
    if (c != end) {
        bool exp_part = false;
        if (*c == '.') {
            c++;
            read = 1;
            while (c != end && is_digit(*c)) {
                const double w = read <= kPow10Max ? pow10[read] : 0.0;
                mantissa = __dadd_rn(mantissa, __dmul_rn((double)(*c - '0'), w));
                read++;
                c++;
            }
            exp_part = c != end && (*c == 'e' || *c == 'E');
        } else {
            exp_part = *c == 'e' || *c == 'E';
        }
        if (exp_part) {
            c++;
            if (c != end && (*c == '+' || *c == '-')) {
                eneg = *c == '-';
                c++;
            } else if (c == end || !is_digit(*c)) {
                return 0.0;
            }
            read = 0;
            while (c != end && is_digit(*c)) {
                exponent = exponent * 10 + (*c - '0');
                c++;
                read++;
            }
            if (eneg) exponent = -exponent;
            if (read == 0) return 0.0;
        }
    }
    double v = mantissa;
    if (exponent) {
        const double p5 = exponent < kPow5Lo ? 0.0
                          : exponent > kPow5Hi ? __longlong_as_double(0x7ff0000000000000ll)
                                               : pow5[exponent - kPow5Lo];
        v = scale2(__dmul_rn(mantissa, p5), exponent);
    }
    return neg ? -v : v;
}

// ParseFloat: blanks skipped, the token ends at a space, tab or '\r' (or the line's end).
__device__ __forceinline__ float parse_float(const char *&t, const char *end, const double *pow5,
                                             const double *pow10) {
    while (t < end && (*t == ' ' || *t == '\t')) t++;
    const char *e = t;
    while (e < end && *e != ' ' && *e != '\t' && *e != '\r') e++;
    const double v = parse_number(t, e, pow5, pow10);
    t = e;
    return __double2float_rn(v);
}

__device__ __forceinline__ void skip_blanks(const char *&t, const char *end) {
    while (t < end && (*t == ' ' || *t == '\t')) t++;
}

// One line: empty, blank or '#' lines are not particles (nor, with the exclusive boundary
// rule, particles whose boundary value is 0); fields in the order position, velocity,
// density, mass, boundary (_SerializerLoadParticles3, :484-531).
__global__ void k_frame_parse(const char *__restrict__ t, size_t bytes, const unsigned *__restrict__ line,
                              unsigned lines, int flags, const double *__restrict__ pow5,
                              const double *__restrict__ pow10, float *__restrict__ vals,
                              unsigned *__restrict__ valid) {
    const unsigned i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= lines) return;
    const char *a = t + line[i];
    const char *stop = t + (i + 1 < lines ? line[i + 1] : bytes);
    const char *end = a;
    while (end < stop && *end != '\n' && *end != '\r' && *end != '\0') end++;   // C-string view
    const char *p = a;
    skip_blanks(p, end);
    bool ok = p < end && *p != '#';
    float f[6] = {0.f, 0.f, 0.f, 0.f, 0.f, 0.f};
    if (ok) {
        if (flags & kFramePosition) {
            for (int k = 0; k < 3; k++) f[k] = parse_float(p, end, pow5, pow10);
            skip_blanks(p, end);
        }
        if (flags & kFrameVelocity) {
            for (int k = 3; k < 6; k++) f[k] = parse_float(p, end, pow5, pow10);
            skip_blanks(p, end);
        }
        if (flags & kFrameDensity) {
            (void)parse_float(p, end, pow5, pow10);
            skip_blanks(p, end);
        }
        if (flags & kFrameMass) {
            (void)parse_float(p, end, pow5, pow10);
            skip_blanks(p, end);
        }
        if (flags & kFrameBoundary) {
            const int b = (int)parse_float(p, end, pow5, pow10);
            if ((flags & kFrameBoundaryExclusive) && !b) ok = false;
        }
    }
    for (int k = 0; k < 6; k++) vals[(size_t)k * lines + i] = f[k];
    valid[i] = ok ? 1u : 0u;
}

__global__ void k_frame_scatter(unsigned lines, int n, const unsigned *__restrict__ valid,
                                const unsigned *__restrict__ index, const float *__restrict__ vals,
                                float *__restrict__ pos, float *__restrict__ vel) {
    const unsigned i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= lines || !valid[i]) return;
    const unsigned q = index[i];
    if ((int)q >= n) return;
    for (int k = 0; k < 3; k++) {
        pos[3 * (size_t)q + k] = vals[(size_t)k * lines + i];
        vel[3 * (size_t)q + k] = vals[(size_t)(k + 3) * lines + i];
    }
}

cudaError_t frame_split_lines(size_t bytes, FrameReadBufs &F, unsigned *lines, unsigned *h_scratch,
                              cudaStream_t s) {
    const size_t chunks = (bytes + kLineChunk - 1) / kLineChunk;
    k_line_count<<<blocks_for((long long)chunks, 256), 256, 0, s>>>(F.text, bytes, F.chunk);
    launch_cell_scan(F.chunk, (unsigned)chunks, F.chunk_part, F.chunk_start, s);
    cudaMemcpyAsync(h_scratch, F.chunk_start + chunks, sizeof(unsigned), cudaMemcpyDeviceToHost, s);
    cudaError_t e = cudaStreamSynchronize(s);
    *lines = *h_scratch;
    return e;
}

cudaError_t frame_parse_lines(size_t bytes, unsigned lines, int flags, FrameReadBufs &F, unsigned *found,
                              unsigned *h_scratch, cudaStream_t s) {
    const size_t chunks = (bytes + kLineChunk - 1) / kLineChunk;
    k_line_write<<<blocks_for((long long)chunks, 256), 256, 0, s>>>(F.text, bytes, F.chunk_start, F.line);
    k_frame_parse<<<blocks_for(lines, 128), 128, 0, s>>>(F.text, bytes, F.line, lines, flags, F.pow5, F.pow10,
                                                         F.vals, F.valid);
    // the scan consumes (zeroes) its input: number the particle lines from a copy of the flags
    cudaMemcpyAsync(F.flag_copy, F.valid, sizeof(unsigned) * lines, cudaMemcpyDeviceToDevice, s);
    launch_cell_scan(F.flag_copy, lines, F.line_part, F.index, s);
    cudaMemcpyAsync(h_scratch, F.index + lines, sizeof(unsigned), cudaMemcpyDeviceToHost, s);
    cudaError_t e = cudaStreamSynchronize(s);
    *found = *h_scratch;
    return e;
}

void launch_frame_scatter(unsigned lines, int n, const FrameReadBufs &F, float *pos, float *vel,
                          cudaStream_t s) {
    k_frame_scatter<<<blocks_for(lines, 256), 256, 0, s>>>(lines, n, F.valid, F.index, F.vals, pos, vel);
}

// ---- host: the fluid section's header (SerializerFindFluidSection, :145-181) ----
namespace {

// ParseFloat's reader on the host (same operations; the host's libm pow / ldexp)
double host_number(const char *s, const char *end) {
    static const double lut[] = {1.0, 0.1, 0.01, 0.001, 0.0001, 0.00001, 0.000001, 0.0000001};
    auto digit = [](char c) { return (unsigned)(c - '0') < 10u; };
    if (s >= end) return 0.0;
    const char *c = s;
    double mantissa = 0.0;
    int exponent = 0, read = 0;
    bool neg = false, eneg = false;
    if (*c == '+' || *c == '-') {
        neg = *c == '-';
        c++;
    } else if (!digit(*c)) {
        return 0.0;
    }
    while (c != end && digit(*c)) {
        mantissa = mantissa * 10.0;
        mantissa = mantissa + (double)(*c - '0');
        c++;
        read++;
    }
    if (read == 0) return 0.0;
    if (c != end) {
        bool exp_part;
        if (*c == '.') {
            c++;
            read = 1;
            while (c != end && digit(*c)) {
                const double w = read < 8 ? lut[read] : std::pow(10.0, -read);
                const double term = (double)(*c - '0') * w;
                mantissa = mantissa + term;
                read++;
                c++;
            }
            exp_part = c != end && (*c == 'e' || *c == 'E');
        } else {
            exp_part = *c == 'e' || *c == 'E';
        }
        if (exp_part) {
            c++;
            if (c != end && (*c == '+' || *c == '-')) {
                eneg = *c == '-';
                c++;
            } else if (c == end || !digit(*c)) {
                return 0.0;
            }
            read = 0;
            while (c != end && digit(*c)) {
                exponent = exponent * 10 + (*c - '0');
                c++;
                read++;
            }
            if (eneg) exponent = -exponent;
            if (read == 0) return 0.0;
        }
    }
    const double v = exponent ? std::ldexp(mantissa * std::pow(5.0, exponent), exponent) : mantissa;
    return neg ? -v : v;
}

float host_float(const char *&t, const char *end) {
    while (t < end && (*t == ' ' || *t == '\t')) t++;
    const char *e = t;
    while (e < end && *e != ' ' && *e != '\t' && *e != '\r') e++;
    const float v = (float)host_number(t, e);
    t = e;
    return v;
}

// SerializerFlagsFromString (:60-81); -1 for an unknown letter
int flags_from(const char *f, size_t len) {
    int flags = 0;
    for (size_t i = 0; i < len; i++) {
        switch (f[i]) {
            case 'p': case 'P': flags |= kFramePosition; break;
            case 'v': case 'V': flags |= kFrameVelocity; break;
            case 'd': case 'D': flags |= kFrameDensity; break;
            case 'm': case 'M': flags |= kFrameMass; break;
            case 'b': case 'B': flags |= kFrameBoundary; break;
            case 'n': case 'N': flags |= 0x10; break;
            case 'l': case 'L': flags |= 0x40; break;
            case 'o': case 'O': flags |= kFrameBoundaryExclusive; break;
            case 'z': case 'Z': flags |= 0x80; break;
            default: return -1;
        }
    }
    return flags;
}

bool next_line(const char *t, size_t len, size_t &pos, size_t &a, size_t &b) {
    if (pos >= len) return false;
    size_t i = pos;
    a = i;
    while (i < len && t[i] != '\n' && t[i] != '\r') i++;
    b = i;
    if (i < len) i += (t[i] == '\r' && i + 1 < len && t[i + 1] == '\n') ? 2 : 1;
    pos = i;
    return true;
}

bool token_is(const char *t, size_t len, const char *word) {
    const size_t wl = strlen(word);
    return len == wl && memcmp(t, word, wl) == 0;
}

}  // namespace

int frame_find_section(const char *text, size_t length, int flags_in, FrameSection *out) {
    size_t at = 0, a = 0, b = 0;
    bool in_region = false, found = false;
    int count = 0;
    const char *fmt = nullptr;
    size_t fmt_len = 0;
    while (!found && next_line(text, length, at, a, b)) {
        size_t ce = a;   // the line as a C string sees it
        while (ce < b && text[ce] != '\0') ce++;
        size_t tok = a;
        // tokens end at a space, tab or NUL; the line's last token is processed with index 0
        for (size_t i = a; i <= b && !found; i++) {
            if (i < b && text[i] != ' ' && text[i] != '\t' && text[i] != '\0') continue;
            const char *t = text + tok;
            const size_t tl = i - tok;
            tok = i + 1;
            if (tl == 0) continue;
            if (!in_region) {
                if (token_is(t, tl, "FluidBegin")) in_region = true;
                continue;
            }
            const char *v = text + (i < b ? i + 1 : a + 1);
            if (token_is(t, tl, "\"Count\"")) {
                while (v < text + ce && (*v == ' ' || *v == '\t')) v++;
                count = (int)host_float(v, text + ce);
            } else if (token_is(t, tl, "\"Format\"")) {
                while (v < text + ce && (*v == ' ' || *v == '\t')) v++;
                fmt = v;
                fmt_len = 0;
                while (v + fmt_len < text + ce && v[fmt_len] != ' ' && v[fmt_len] != '\t') fmt_len++;
            } else if (token_is(t, tl, "DataBegin")) {
                found = true;
            } else if (token_is(t, tl, "FluidEnd")) {
                in_region = false;
            }
        }
    }
    int flags = flags_in;
    if (fmt && fmt_len > 0) {
        flags = flags_from(fmt, fmt_len);
        if (flags < 0) return 1;
    }
    if (!found) return 2;
    // the data ends at the first line holding "DataEnd" that is not a comment
    // (_SerializerLoadParticles3, :471-482)
    const size_t begin = at;
    size_t from = begin;
    for (;;) {
        const char *p = nullptr;
        for (size_t k = from; k + 7 <= length; k++) {
            const void *q = memchr(text + k, 'D', length - 7 - k + 1);
            if (!q) break;
            k = (size_t)((const char *)q - text);
            if (memcmp(text + k, "DataEnd", 7) == 0) {
                p = text + k;
                break;
            }
        }
        if (!p) return 2;
        size_t ls = (size_t)(p - text);
        while (ls > begin && text[ls - 1] != '\n' && text[ls - 1] != '\r') ls--;
        size_t q = ls;
        while (q < (size_t)(p - text) && (text[q] == ' ' || text[q] == '\t')) q++;
        bool cut = false;   // a NUL before it hides "DataEnd" from the reference's string view
        for (size_t r = ls; r < (size_t)(p - text); r++) cut = cut || text[r] == '\0';
        if (text[q] != '#' && !cut) {
            out->data_begin = begin;
            out->data_end = ls;
            out->count = count;
            out->flags = flags;
            return 0;
        }
        from = (size_t)(p - text) + 7;
    }
}

}  // namespace bbg
