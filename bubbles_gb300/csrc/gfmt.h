// gfmt.h -- C printf "%g" of a float value (promoted to double), exactly, on the host and
// on the device.
//
// The reference's particle frames print every value with fprintf("%g")
// (src/third/serializer.cpp:20-45): six significant digits, correctly rounded (ties to
// even) from the exact binary value, then %e or %f style by the decimal exponent, trailing
// zeros removed.  A float is m * 2^e with m < 2^24, so the six digits are
// q = round(m * 2^e * 10^s) for s = 5 - X, X the decimal exponent.  q is computed exactly
// as floor(A / B) with A = m * 2^max(e,0) * 10^max(s,0) and B = 2^max(-e,0) * 10^max(-s,0)
// in 32-bit limbs (A < 2^192, B < 2^160), q (< 2^20) found bit by bit, and the remainder
// decides the rounding.
#pragma once

#include <stdint.h>

#if defined(__CUDACC__)
#define GFMT_FN __host__ __device__ __forceinline__
#else
#define GFMT_FN inline
#endif

namespace gfmt {

constexpr int kLimbs = 7;   // 224 bits

struct Big {
    uint32_t w[kLimbs];
};

GFMT_FN void big_set(Big &a, uint64_t v) {
    for (int i = 0; i < kLimbs; i++) a.w[i] = 0;
    a.w[0] = (uint32_t)v;
    a.w[1] = (uint32_t)(v >> 32);
}

GFMT_FN void big_mul_small(Big &a, uint32_t f) {
    uint64_t carry = 0;
    for (int i = 0; i < kLimbs; i++) {
        const uint64_t t = (uint64_t)a.w[i] * f + carry;
        a.w[i] = (uint32_t)t;
        carry = t >> 32;
    }
}

GFMT_FN void big_shl(Big &a, int bits) {
    const int words = bits >> 5, r = bits & 31;
    for (int i = kLimbs - 1; i >= 0; i--) {
        uint32_t v = 0;
        const int src = i - words;
        if (src >= 0) {
            v = a.w[src] << r;
            if (r && src - 1 >= 0) v |= a.w[src - 1] >> (32 - r);
        }
        a.w[i] = v;
    }
}

GFMT_FN int big_cmp(const Big &a, const Big &b) {
    for (int i = kLimbs - 1; i >= 0; i--) {
        if (a.w[i] != b.w[i]) return a.w[i] < b.w[i] ? -1 : 1;
    }
    return 0;
}

GFMT_FN void big_sub(Big &a, const Big &b) {   // a -= b (a >= b)
    int64_t borrow = 0;
    for (int i = 0; i < kLimbs; i++) {
        const int64_t t = (int64_t)a.w[i] - (int64_t)b.w[i] - borrow;
        a.w[i] = (uint32_t)t;
        borrow = t < 0 ? 1 : 0;
    }
}

// Six significant digits of m * 2^e at decimal exponent X: q = A / B rounded half to even.
// Returns q (may be 10^6 after rounding up, or outside [10^5, 10^6) if X is wrong).
GFMT_FN uint32_t digits6(uint32_t m, int e, int X) {
    const int s = 5 - X;
    Big A, B;
    big_set(A, m);
    big_set(B, 1);
    for (int k = 0; k < s; k++) big_mul_small(A, 10);
    for (int k = 0; k < -s; k++) big_mul_small(B, 10);
    if (e > 0) big_shl(A, e);
    if (e < 0) big_shl(B, -e);
    // q = floor(A / B) < 2^21, bit by bit
    uint32_t q = 0;
    Big prod;
    for (int bit = 20; bit >= 0; bit--) {
        const uint32_t cand = q | (1u << bit);
        prod = B;
        big_mul_small(prod, cand);
        if (big_cmp(prod, A) <= 0) q = cand;
    }
    // remainder r = A - q B; round: 2r vs B
    prod = B;
    big_mul_small(prod, q);
    Big r = A;
    big_sub(r, prod);
    big_shl(r, 1);
    const int c = big_cmp(r, B);
    if (c > 0 || (c == 0 && (q & 1u))) q += 1;
    return q;
}

// Writes printf("%g", (double)f) into out (at most 14 bytes, no terminator); returns the
// length.
GFMT_FN int format_g(float f, char *out) {
    uint32_t bits;
    {
        union {
            float f;
            uint32_t u;
        } cv;
        cv.f = f;
        bits = cv.u;
    }
    int len = 0;
    const bool neg = (bits >> 31) != 0;
    const uint32_t ex = (bits >> 23) & 0xffu, frac = bits & 0x7fffffu;
    if (ex == 0xffu) {
        if (frac) {   // glibc prints the sign of a NaN
            if (neg) out[len++] = '-';
            out[len++] = 'n'; out[len++] = 'a'; out[len++] = 'n';
        } else {
            if (neg) out[len++] = '-';
            out[len++] = 'i'; out[len++] = 'n'; out[len++] = 'f';
        }
        return len;
    }
    if (neg) out[len++] = '-';
    if (ex == 0 && frac == 0) {
        out[len++] = '0';
        return len;
    }
    uint32_t m;
    int e;
    if (ex == 0) {
        m = frac;
        e = -149;
    } else {
        m = frac | 0x800000u;
        e = (int)ex - 150;
    }
    // decimal exponent estimate from the binary one: log10(m 2^e) ~ (bits(m) - 1 + e) log10 2
    int msb = 31;
    while (!(m >> msb)) msb--;
    int X = (int)((double)(msb + e) * 0.30102999566398120);
    if ((double)(msb + e) * 0.30102999566398120 < (double)X) X--;   // floor for negatives
    uint32_t q = digits6(m, e, X);
    for (int guard = 0; guard < 4 && (q < 100000u || q >= 1000000u); guard++) {
        if (q >= 1000000u) {
            // either X too small, or rounding carried to 10^6
            const uint32_t q2 = digits6(m, e, X + 1);
            if (q2 >= 100000u && q2 < 1000000u) {
                X += 1;
                q = q2;
            } else if (q2 == 1000000u) {
                X += 2;
                q = 100000u;
            } else {
                X += 1;
                q = q2;
            }
        } else {
            X -= 1;
            q = digits6(m, e, X);
        }
    }
    char d[6];
    for (int k = 5; k >= 0; k--) {
        d[k] = (char)('0' + q % 10u);
        q /= 10u;
    }
    int nd = 6;   // significant digits kept after removing trailing zeros
    while (nd > 1 && d[nd - 1] == '0') nd--;
    if (X < -4 || X >= 6) {
        out[len++] = d[0];
        if (nd > 1) {
            out[len++] = '.';
            for (int k = 1; k < nd; k++) out[len++] = d[k];
        }
        out[len++] = 'e';
        int ax = X;
        if (ax < 0) {
            out[len++] = '-';
            ax = -ax;
        } else {
            out[len++] = '+';
        }
        if (ax >= 100) {
            out[len++] = (char)('0' + ax / 100);
            ax %= 100;
            out[len++] = (char)('0' + ax / 10);
            out[len++] = (char)('0' + ax % 10);
        } else {
            out[len++] = (char)('0' + ax / 10);
            out[len++] = (char)('0' + ax % 10);
        }
        return len;
    }
    if (X >= 0) {
        // integer part: digits 0..X, fraction: X+1..nd-1
        for (int k = 0; k <= X; k++) out[len++] = k < 6 ? d[k] : '0';
        if (nd > X + 1) {
            out[len++] = '.';
            for (int k = X + 1; k < nd; k++) out[len++] = d[k];
        }
        return len;
    }
    // X in [-4, -1]: 0.000ddd
    out[len++] = '0';
    out[len++] = '.';
    for (int k = 0; k < -X - 1; k++) out[len++] = '0';
    for (int k = 0; k < nd; k++) out[len++] = d[k];
    return len;
}

}  // namespace gfmt
