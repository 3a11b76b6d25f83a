// dev_decode.cu -- request bodies of POST /nearest decoded on the device.
//
// nearest_handler_callback (src/compare_handler.c:300-390) parses the body
// with cJSON, checks that the parsed value has exactly db_vector_size
// children and that each is a number, and copies each number's valuedouble.
// cJSON (a third-party library the reference links, version not pinned; the
// rules below are those of the published cJSON 1.7 sources) reads a number
// by collecting the run of characters in [0-9+-eE.] (at most 63) and calling
// strtod on it, advancing by what strtod consumed; the value is therefore
// the correctly rounded double of the decimal that strtod accepts.
//
// A body that is a flat array of numbers (the request a client sends) is
// decoded by one warp: each lane classifies 16 bytes per step, a warp scan
// carries the previous token and the number count across lanes, and each
// lane converts the numbers that start in its bytes.  Every other body
// (objects, strings, nesting, a NUL or a byte-order mark before the closing
// bracket, ...) goes to the general path: one thread per body validates the
// whole JSON text with cJSON's grammar (whitespace = any byte <= 32; a UTF-8
// byte-order mark is skipped; nesting up to 1000; strings with cJSON's escape
// rules; literals null / true / false; content after the value is ignored; a
// NUL byte ends the text) and records where each top-level child starts and
// whether it is a number, then one thread per (body, child) converts it.
// A number is converted exactly:
//   - w x 10^q with w < 2^53 and |q| <= 22: one correctly rounded IEEE
//     multiply or divide (both operands exact: Clinger's fast path);
//   - otherwise, for -342 <= q <= 308, the Eisel-Lemire step (D. Lemire,
//     "Number Parsing at a Gigabyte per Second", 2021): w, normalised to 64
//     bits, times the 128-bit truncated significand of 5^q gives the 54
//     leading bits and enough of the rest to prove the rounding, unless a
//     carry or a tie cannot be excluded (or the result is subnormal);
//   - what that step leaves undecided: exact big-integer arithmetic: w x 10^q rounded to 53 bits
//     (q >= 0), or the quotient w x 2^s / 10^-q taken to 54+ bits with a
//     sticky remainder (q < 0), rounded half to even, with subnormals and
//     overflow to infinity as strtod gives them;
//   - more than 19 significant digits: w = the first 19 digits and w + 1
//     bound the value; if both round to the same double that is the result,
//     else every digit strtod consumed (at most 62) goes into the exact
//     big-integer rounding.
#include <algorithm>
#include <cstring>
#include <mutex>
#include <new>
#include <vector>

#include "dev_common.cuh"
#include "dev_store.cuh"

namespace svdb {
namespace {

constexpr int kMaxDepth = 1000;  // CJSON_NESTING_LIMIT
constexpr int kLimbs = 22;       // 1408 bits: 10^400 and 2^56 x 10^343 fit

__device__ __forceinline__ bool is_num_char(uint8_t c) {
    return (c >= '0' && c <= '9') || c == '+' || c == '-' || c == 'e' || c == 'E' || c == '.';
}

// ---- strtod's syntax on cJSON's run -------------------------------------------
struct Dec {
    uint64_t w;     // first (up to) 19 significant digits
    int64_t q;      // decimal exponent of w's last digit
    bool neg;
    bool more;      // significant digits beyond the 19 kept
    bool zero;      // every digit is 0
};

// Parses the number at p[0..n) the way strtod parses cJSON's run of number
// characters; returns the characters consumed (0: no number) and the run's
// length (at most 63) in *run_out.
__device__ int scan_number(const uint8_t* p, int n, Dec& d, int* run_out = nullptr) {
    int run = 0;
    while (run < n && run < 63 && is_num_char(p[run])) ++run;
    if (run_out) *run_out = run;
    int i = 0;
    d.neg = false;
    if (i < run && (p[i] == '+' || p[i] == '-')) {
        d.neg = p[i] == '-';
        ++i;
    }
    uint64_t w = 0;
    int kept = 0;
    int64_t dropped_int = 0;  // integer digits beyond the kept ones
    int64_t frac_kept = 0;    // fraction digits inside w
    bool more = false, any = false, nonzero = false;
    while (i < run && p[i] >= '0' && p[i] <= '9') {
        any = true;
        const int dg = p[i] - '0';
        if (w == 0 && dg == 0) {
            // leading zero
        } else if (kept < 19) {
            w = w * 10 + dg;
            ++kept;
            nonzero = true;
        } else {
            ++dropped_int;
            more |= dg != 0;
            nonzero = true;
        }
        ++i;
    }
    if (i < run && p[i] == '.') {
        int j = i + 1;
        bool fany = false;
        while (j < run && p[j] >= '0' && p[j] <= '9') {
            fany = true;
            const int dg = p[j] - '0';
            if (w == 0 && dg == 0) {
                ++frac_kept;  // leading zeros after the point scale the value
            } else if (kept < 19) {
                w = w * 10 + dg;
                ++kept;
                ++frac_kept;
                nonzero = true;
            } else {
                more |= dg != 0;
            }
            ++j;
        }
        if (any || fany) {
            any = true;
            i = j;
        }
    }
    if (!any) return 0;
    int64_t e = 0;
    if (i < run && (p[i] == 'e' || p[i] == 'E')) {
        int j = i + 1;
        bool eneg = false;
        if (j < run && (p[j] == '+' || p[j] == '-')) {
            eneg = p[j] == '-';
            ++j;
        }
        if (j < run && p[j] >= '0' && p[j] <= '9') {
            while (j < run && p[j] >= '0' && p[j] <= '9') {
                if (e < 100000000) e = e * 10 + (p[j] - '0');
                ++j;
            }
            if (eneg) e = -e;
            i = j;
        }
    }
    d.w = w;
    d.q = e + dropped_int - frac_kept;
    d.more = more;
    d.zero = !nonzero;
    return i;
}

// ---- big integers (little-endian 64-bit limbs) --------------------------------
struct Big {
    uint64_t v[kLimbs];
    int n;  // limbs in use
};

__device__ __forceinline__ void big_set(Big& b, uint64_t x) {
    b.v[0] = x;
    b.n = x ? 1 : 0;
}

__device__ __forceinline__ void big_mul_small(Big& b, uint64_t m) {
    uint64_t carry = 0;
    for (int i = 0; i < b.n; ++i) {
        const uint64_t lo = b.v[i] * m;
        const uint64_t hi = __umul64hi(b.v[i], m);
        const uint64_t s = lo + carry;
        carry = hi + (s < lo ? 1 : 0);
        b.v[i] = s;
    }
    if (carry && b.n < kLimbs) b.v[b.n++] = carry;
}

__device__ __forceinline__ void big_pow10(Big& b, int64_t k) {  // b *= 10^k
    const uint64_t p19 = 10000000000000000000ull;
    while (k >= 19) {
        big_mul_small(b, p19);
        k -= 19;
    }
    uint64_t m = 1;
    while (k-- > 0) m *= 10;
    if (m > 1) big_mul_small(b, m);
}

__device__ __forceinline__ void big_add_small(Big& b, uint64_t a) {
    for (int i = 0; i < b.n && a; ++i) {
        const uint64_t s = b.v[i] + a;
        a = s < a ? 1 : 0;
        b.v[i] = s;
    }
    if (a && b.n < kLimbs) b.v[b.n++] = a;
}

__device__ __forceinline__ void big_pow5(Big& b, int64_t k) {  // b *= 5^k
    const uint64_t p27 = 7450580596923828125ull;                  // 5^27 < 2^63
    while (k >= 27) {
        big_mul_small(b, p27);
        k -= 27;
    }
    uint64_t m = 1;
    while (k-- > 0) m *= 5;
    if (m > 1) big_mul_small(b, m);
}

__device__ __forceinline__ int big_bits(const Big& b) {
    if (b.n == 0) return 0;
    return (b.n - 1) * 64 + (64 - __clzll((long long)b.v[b.n - 1]));
}

__device__ __forceinline__ int big_bit(const Big& b, int k) {  // bit k (0 beyond the top)
    const int l = k >> 6;
    return l < b.n ? (int)((b.v[l] >> (k & 63)) & 1u) : 0;
}

__device__ __forceinline__ bool big_any_below(const Big& b, int k) {  // any set bit below bit k?
    const int l = k >> 6;
    for (int i = 0; i < l && i < b.n; ++i)
        if (b.v[i]) return true;
    if (l < b.n && (k & 63)) return (b.v[l] & ((1ull << (k & 63)) - 1)) != 0;
    return false;
}

__device__ __forceinline__ void big_shl(Big& b, int s) {
    const int ls = s >> 6, bs = s & 63;
    const int nn = min(kLimbs, b.n + ls + 1);
    for (int i = nn - 1; i >= 0; --i) {
        const int src = i - ls;
        uint64_t x = 0;
        if (src >= 0 && src < b.n) x = b.v[src] << bs;
        if (bs && src - 1 >= 0 && src - 1 < b.n) x |= b.v[src - 1] >> (64 - bs);
        b.v[i] = x;
    }
    b.n = nn;
    while (b.n > 0 && b.v[b.n - 1] == 0) --b.n;
}

// a >= d << k ?  (d << k compared limb by limb without forming it)
__device__ __forceinline__ uint64_t shl_limb(const Big& d, int k, int i) {
    const int ls = k >> 6, bs = k & 63;
    const int src = i - ls;
    uint64_t x = 0;
    if (src >= 0 && src < d.n) x = d.v[src] << bs;
    if (bs && src - 1 >= 0 && src - 1 < d.n) x |= d.v[src - 1] >> (64 - bs);
    return x;
}

__device__ bool big_ge_shl(const Big& a, const Big& d, int k) {
    const int top = max(a.n, d.n + (k >> 6) + 1);
    for (int i = top - 1; i >= 0; --i) {
        const uint64_t x = i < a.n ? a.v[i] : 0, y = shl_limb(d, k, i);
        if (x != y) return x > y;
    }
    return true;
}

__device__ void big_sub_shl(Big& a, const Big& d, int k) {  // a -= d << k (a >= d << k)
    uint64_t borrow = 0;
    for (int i = 0; i < a.n; ++i) {
        const uint64_t y = shl_limb(d, k, i);
        const uint64_t t = a.v[i] - y;
        const uint64_t b1 = a.v[i] < y ? 1 : 0;
        const uint64_t t2 = t - borrow;
        const uint64_t b2 = t < borrow ? 1 : 0;
        a.v[i] = t2;
        borrow = b1 | b2;
    }
    while (a.n > 0 && a.v[a.n - 1] == 0) --a.n;
}

// Round m (exact binary value m_int x 2^e2 given as: `bits` = the integer's
// top-bit index, accessor through a Big) -- assembled by the callers below.
__device__ __forceinline__ double make_double(uint64_t mant, int64_t e2, bool neg) {
    // mant in [2^52, 2^53) for normals with value mant x 2^e2, or < 2^52 for subnormals (e2 = -1074)
    if (mant == 0) return neg ? -0.0 : 0.0;
    if (e2 + 52 > 1023) return neg ? -__longlong_as_double(0x7ff0000000000000ll) : __longlong_as_double(0x7ff0000000000000ll);
    uint64_t bits;
    if (mant < (1ull << 52)) {
        bits = mant;  // subnormal (e2 == -1074)
    } else {
        bits = ((uint64_t)(e2 + 52 + 1023) << 52) | (mant & ((1ull << 52) - 1));
    }
    if (neg) bits |= 0x8000000000000000ull;
    return __longlong_as_double((long long)bits);
}

// Round the exact value X x 2^-s (X a big integer, sticky = nonzero bits
// below X) to a double, half to even.
__device__ double round_big(const Big& X, int64_t s, bool sticky_in, bool neg) {
    const int nb = big_bits(X);
    if (nb == 0) return neg ? -0.0 : 0.0;
    const int64_t top = nb - 1 - s;  // exponent of the leading bit
    // drop = bits below the 53-bit mantissa (or below 2^-1074 for subnormals)
    int64_t drop = nb - 53;
    if (top < -1022) drop = nb - 53 + (-1022 - top);
    if (drop > nb + 1) return neg ? -0.0 : 0.0;  // below half of the least subnormal
    uint64_t mant = 0;
    bool half = false, rest = sticky_in;
    if (drop <= 0) {
        for (int k = nb - 1; k >= 0; --k) mant = (mant << 1) | (uint64_t)big_bit(X, k);
        mant <<= -drop;
    } else {
        for (int64_t k = nb - 1; k >= drop; --k) mant = (mant << 1) | (uint64_t)big_bit(X, (int)k);
        half = big_bit(X, (int)(drop - 1)) != 0;
        rest = rest || big_any_below(X, (int)(drop - 1));
    }
    if (half && (rest || (mant & 1))) ++mant;
    int64_t e2 = drop - s;  // value = mant x 2^e2; below 2^52 only for subnormals (e2 = -1074)
    if (mant == (1ull << 53)) {
        mant >>= 1;
        ++e2;
    }
    return make_double(mant, e2, neg);
}

// exact w x 10^q (w > 0) rounded to double
__device__ double exact_value(uint64_t w, int64_t q, bool neg) {
    if (q > 310) return neg ? -__longlong_as_double(0x7ff0000000000000ll) : __longlong_as_double(0x7ff0000000000000ll);
    if (q < -345) return neg ? -0.0 : 0.0;  // w < 10^19: below 10^-326, under half of the least subnormal
    if (q >= 0) {
        Big X;
        big_set(X, w);
        big_pow10(X, q);
        return round_big(X, 0, false, neg);
    }
    Big D;
    big_set(D, 1);
    big_pow10(D, -q);
    // quotient Q of w x 2^s by D, at least 2^55 (56 bits) and below 2^62:
    // s = max(0, bits(D) - bits(w) + 56)
    const int wb = 64 - __clzll((long long)w);
    int64_t s = (int64_t)big_bits(D) - wb + 56;
    if (s < 0) s = 0;
    Big A;
    big_set(A, w);
    if (s > 0) big_shl(A, (int)s);
    uint64_t Q = 0;
    for (int k = 63; k >= 0; --k) {
        if (big_ge_shl(A, D, k)) {
            big_sub_shl(A, D, k);
            Q |= 1ull << k;
        }
    }
    Big QB;
    big_set(QB, Q);
    return round_big(QB, s, A.n != 0, neg);
}

// ---- the Eisel-Lemire step ----------------------------------------------------
constexpr int kP5Min = -342, kP5Max = 308;  // 10^-343 x (10^19 - 1) < half the least subnormal; 10^309 > DBL_MAX
// 5^q = (T + f) x 2^e with T = g_p5[q - kP5Min] in [2^127, 2^128) (x: high, y: low 64 bits),
// e = g_p5e[q - kP5Min] and 0 <= f < 1 (f = 0 exactly for 0 <= q <= 55, where 5^q < 2^128)
__device__ ulonglong2 g_p5[kP5Max - kP5Min + 1];
__device__ int32_t g_p5e[kP5Max - kP5Min + 1];

// The table, once per context, by exact big-integer arithmetic:
// q >= 0: T = floor(5^q / 2^(b - 128)), b = bits(5^q) (a left shift when b < 128);
// q < 0:  T = floor(2^(b + 127) / 5^-q), b = bits(5^-q) (5^-q is not a power of two,
//         so 2^(b + 127) / 5^-q lies strictly between 2^127 and 2^128).
__global__ void k_pow5_init() {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i > kP5Max - kP5Min) return;
    const int q = i + kP5Min;
    uint64_t hi = 0, lo = 0;
    int e;
    if (q >= 0) {
        Big X;
        big_set(X, 1);
        big_pow5(X, q);
        const int s = big_bits(X) - 128;
        for (int k = 127; k >= 0; --k) {
            const int src = k + s;
            const uint64_t bit = src >= 0 ? (uint64_t)big_bit(X, src) : 0;
            if (k >= 64) hi |= bit << (k - 64);
            else lo |= bit << k;
        }
        e = s;
    } else {
        Big D, A;
        big_set(D, 1);
        big_pow5(D, -q);
        const int k = big_bits(D) + 127;
        big_set(A, 1);
        big_shl(A, k);
        for (int j = 127; j >= 0; --j)
            if (big_ge_shl(A, D, j)) {
                big_sub_shl(A, D, j);
                if (j >= 64) hi |= 1ull << (j - 64);
                else lo |= 1ull << j;
            }
        e = -k;
    }
    g_p5[i] = make_ulonglong2(hi, lo);
    g_p5e[i] = e;
}

// w x 10^q (w != 0) correctly rounded, when the 192-bit product decides it;
// false: undecided here (exact_value decides).
//
// wn = w << l (top bit set), P = wn x T.  The exact value is (P + wn f) x
// 2^(e + q - l) with 0 <= wn f < 2^64, so the bits of P from bit 64 up are
// exact up to a carry of one into bit 64.  P's top bit is bit 190 or 191; the
// 53 bits below it with it are the mantissa, the next the round bit, and the
// bits between it and bit 64 (the "field") decide: a field of all ones lets a
// carry reach the round bit (undecided); a round bit of 1 with a non-zero
// field rounds up; with a zero field it is a tie only if the lower bits are
// zero too, known only when f = 0 (0 <= q <= 55).
__device__ bool el_value(uint64_t w, int64_t q, bool neg, double* out) {
    if (q < kP5Min || q > kP5Max) return false;
    const ulonglong2 T = g_p5[q - kP5Min];
    const int64_t ep = g_p5e[q - kP5Min];
    const int l = __clzll((long long)w);
    const uint64_t wn = w << l;
    const uint64_t a_lo = wn * T.x, a_hi = __umul64hi(wn, T.x);
    const uint64_t b_lo = wn * T.y, b_hi = __umul64hi(wn, T.y);
    const uint64_t p1 = a_lo + b_hi;
    const uint64_t p2 = a_hi + (p1 < a_lo ? 1 : 0);
    const uint64_t p0 = b_lo;
    const int top = (int)(p2 >> 63);  // P's top bit: 190 + top
    const int sh = 9 + top;           // bits of p2 below the 54 kept
    const uint64_t fmask = (1ull << sh) - 1;
    const uint64_t f_hi = p2 & fmask;
    if (f_hi == fmask && p1 == ~0ull) return false;
    const uint64_t m54 = p2 >> sh;
    uint64_t m = m54 >> 1;
    if (m54 & 1) {
        const bool field_zero = f_hi == 0 && p1 == 0;
        if (field_zero && !(q >= 0 && q <= 55)) return false;
        if (!field_zero || p0 != 0 || (m & 1)) ++m;
    }
    int64_t E = 190 + top + ep + q - l;  // the value is m x 2^(E - 52)
    if (m == (1ull << 53)) {
        m >>= 1;
        ++E;
    }
    if (E < -1022) return false;  // subnormal: exact_value
    if (E > 1023) {
        *out = neg ? -__longlong_as_double(0x7ff0000000000000ll) : __longlong_as_double(0x7ff0000000000000ll);
        return true;
    }
    uint64_t bits = ((uint64_t)(E + 1023) << 52) | (m & ((1ull << 52) - 1));
    if (neg) bits |= 0x8000000000000000ull;
    *out = __longlong_as_double((long long)bits);
    return true;
}

__device__ __forceinline__ double value_of(uint64_t w, int64_t q, bool neg) {
    double v;
    return el_value(w, q, neg, &v) ? v : exact_value(w, q, neg);
}

// exact W x 10^q (W > 0, nd significant digits; W is consumed) rounded to double
__device__ double exact_big(Big& W, int nd, int64_t q, bool neg) {
    if (nd + q <= -324) return neg ? -0.0 : 0.0;  // below 10^-324: under half the least subnormal
    if (nd - 1 + q >= 309) return neg ? -__longlong_as_double(0x7ff0000000000000ll) : __longlong_as_double(0x7ff0000000000000ll);
    if (q >= 0) {
        big_pow10(W, q);  // below 10^309: 1,027 bits
        return round_big(W, 0, false, neg);
    }
    Big D;  // 10^-q, -q < nd + 324 <= 386: 1,286 bits at most
    big_set(D, 1);
    big_pow10(D, -q);
    int64_t s = (int64_t)big_bits(D) - big_bits(W) + 56;  // the quotient gets at least 56 bits
    if (s < 0) s = 0;
    if (s > 0) big_shl(W, (int)s);
    Big Q;
    const int kq = big_bits(W) - big_bits(D);  // the quotient is below 2^(kq + 1)
    Q.n = kq / 64 + 1;
    for (int i = 0; i < Q.n; ++i) Q.v[i] = 0;
    for (int k = kq; k >= 0; --k)
        if (big_ge_shl(W, D, k)) {
            big_sub_shl(W, D, k);
            Q.v[k >> 6] |= 1ull << (k & 63);
        }
    while (Q.n > 0 && Q.v[Q.n - 1] == 0) --Q.n;
    return round_big(Q, s, W.n != 0, neg);
}

// the number strtod consumed, p[0..used), with every digit
__device__ double exact_text(const uint8_t* p, int used) {
    int i = 0;
    bool neg = false;
    if (i < used && (p[i] == '+' || p[i] == '-')) {
        neg = p[i] == '-';
        ++i;
    }
    Big W;
    W.n = 0;
    int nd = 0;
    int64_t q = 0;
    for (bool frac = false; i < used; ++i) {
        if (p[i] == '.' && !frac) {
            frac = true;
            continue;
        }
        if (p[i] < '0' || p[i] > '9') break;
        const uint64_t dg = p[i] - '0';
        if (W.n != 0 || dg != 0) {
            big_mul_small(W, 10);
            big_add_small(W, dg);
            ++nd;
        }
        if (frac) --q;
    }
    if (i < used && (p[i] == 'e' || p[i] == 'E')) {
        ++i;
        bool eneg = false;
        if (i < used && (p[i] == '+' || p[i] == '-')) {
            eneg = p[i] == '-';
            ++i;
        }
        int64_t e = 0;
        for (; i < used && p[i] >= '0' && p[i] <= '9'; ++i)
            if (e < 100000000) e = e * 10 + (p[i] - '0');
        q += eneg ? -e : e;
    }
    if (W.n == 0) return neg ? -0.0 : 0.0;
    return exact_big(W, nd, q, neg);
}

// the correctly rounded double of the number strtod consumed, p[0..used), scanned into d
__device__ double to_double(const Dec& d, const uint8_t* p, int used) {
    if (d.zero || d.w == 0) return d.neg ? -0.0 : 0.0;
    if (!d.more) {
        if (d.w <= (1ull << 53) && d.q >= -22 && d.q <= 22) {
            double p = 1.0;
            for (int k = 0; k < (d.q < 0 ? -d.q : d.q); ++k) p *= 10.0;  // 10^k, k <= 22: exact
            const double x = (double)d.w;
            const double v = d.q >= 0 ? __dmul_rn(x, p) : __ddiv_rn(x, p);
            return d.neg ? -v : v;
        }
        return value_of(d.w, d.q, d.neg);
    }
    // digits beyond the 19 kept: the value lies strictly between w and w + 1 units
    const double a = value_of(d.w, d.q, d.neg);
    const double b = value_of(d.w + 1, d.q, d.neg);
    if (__double_as_longlong(a) == __double_as_longlong(b)) return a;
    return exact_text(p, used);
}

// ---- cJSON's grammar, one thread per body ---------------------------------------
struct Cursor {
    const uint8_t* p;
    int64_t n;
    int64_t i;
};

__device__ __forceinline__ void skip_ws(Cursor& c) {
    while (c.i < c.n && c.p[c.i] <= 32) ++c.i;
}

__device__ __forceinline__ int hexval(uint8_t c) {
    if (c >= '0' && c <= '9') return c - '0';
    if (c >= 'A' && c <= 'F') return 10 + c - 'A';
    if (c >= 'a' && c <= 'f') return 10 + c - 'a';
    return -1;
}

__device__ __forceinline__ unsigned hex4(const uint8_t* s) {  // cJSON's parse_hex4: 0 on a bad digit
    unsigned h = 0;
    for (int k = 0; k < 4; ++k) {
        const int v = hexval(s[k]);
        if (v < 0) return 0;
        h = (h << 4) | (unsigned)v;
    }
    return h;
}

// a string at c.i (which holds '"'); cJSON's parse_string
__device__ bool parse_string(Cursor& c) {
    int64_t e = c.i + 1;
    while (e < c.n && c.p[e] != '"') {
        if (c.p[e] == '\\') {
            if (e + 1 >= c.n) return false;
            ++e;
        }
        ++e;
    }
    if (e >= c.n) return false;  // no closing quote
    for (int64_t k = c.i + 1; k < e;) {
        if (c.p[k] != '\\') {
            ++k;
            continue;
        }
        if (e - k < 1) return false;
        const uint8_t x = c.p[k + 1];
        if (x == 'b' || x == 'f' || x == 'n' || x == 'r' || x == 't' || x == '"' || x == '\\' || x == '/') {
            k += 2;
        } else if (x == 'u') {
            if (e - k < 6) return false;
            const unsigned first = hex4(c.p + k + 2);
            if (first >= 0xDC00 && first <= 0xDFFF) return false;
            if (first >= 0xD800 && first <= 0xDBFF) {
                const int64_t s2 = k + 6;
                if (e - s2 < 6) return false;
                if (c.p[s2] != '\\' || c.p[s2 + 1] != 'u') return false;
                const unsigned second = hex4(c.p + s2 + 2);
                if (second < 0xDC00 || second > 0xDFFF) return false;
                k += 12;
            } else {
                k += 6;
            }
        } else {
            return false;
        }
    }
    c.i = e + 1;
    return true;
}

__device__ __forceinline__ bool lit(const Cursor& c, const char* s, int len) {
    if (c.n - c.i < len) return false;
    for (int k = 0; k < len; ++k)
        if (c.p[c.i + k] != (uint8_t)s[k]) return false;
    return true;
}

// Validates the body and records its top-level children (first `cap` of
// them): offset of a number child, or -1 for any other kind.  Returns the
// children count, or -1 for text cJSON rejects.
__device__ int64_t parse_body(const uint8_t* p, int64_t n, int64_t* child, int64_t cap) {
    Cursor c{p, n, 0};
    for (int64_t k = 0; k < n; ++k)  // a NUL ends the text
        if (p[k] == 0) {
            c.n = k;
            break;
        }
    if (c.n >= 4 && p[0] == 0xEF && p[1] == 0xBB && p[2] == 0xBF) c.i = 3;  // cJSON skips a UTF-8 BOM
    // container stack: bit = 1 for an object; depth 0 = the top-level value
    uint32_t stk[(kMaxDepth + 31) / 32 + 1];
    int depth = 0;
    int64_t count = 0;
    skip_ws(c);
    bool top_container = false;
    bool expect_value = true;
    for (;;) {
        if (expect_value) {
            // a value at c.i (whitespace already skipped)
            if (c.i >= c.n) return -1;
            const uint8_t ch = c.p[c.i];
            const bool at_top_child = top_container && depth == 1;
            if (ch == '[' || ch == '{') {
                if (depth >= kMaxDepth) return -1;
                const bool obj = ch == '{';
                if (obj)
                    stk[depth >> 5] |= 1u << (depth & 31);
                else
                    stk[depth >> 5] &= ~(1u << (depth & 31));
                if (at_top_child) {
                    if (count < cap) child[count] = -1;
                    ++count;
                }
                if (depth == 0) top_container = true;
                ++depth;
                ++c.i;
                skip_ws(c);
                if (c.i < c.n && c.p[c.i] == (obj ? '}' : ']')) {  // empty container
                    ++c.i;
                    --depth;
                    expect_value = false;
                } else if (obj) {
                    if (c.i >= c.n || c.p[c.i] != '"' || !parse_string(c)) return -1;
                    skip_ws(c);
                    if (c.i >= c.n || c.p[c.i] != ':') return -1;
                    ++c.i;
                    skip_ws(c);
                }
                if (expect_value) continue;
            } else {
                int64_t start = c.i;
                bool number = false;
                if (ch == '"') {
                    if (!parse_string(c)) return -1;
                } else if (lit(c, "null", 4)) {
                    c.i += 4;
                } else if (lit(c, "false", 5)) {
                    c.i += 5;
                } else if (lit(c, "true", 4)) {
                    c.i += 4;
                } else if (ch == '-' || (ch >= '0' && ch <= '9')) {
                    Dec d;
                    const int used = scan_number(c.p + c.i, c.n - c.i < 64 ? (int)(c.n - c.i) : 64, d);
                    if (used == 0) return -1;
                    c.i += used;
                    number = true;
                } else {
                    return -1;
                }
                if (at_top_child) {
                    if (count < cap) child[count] = number ? start : -1;
                    ++count;
                }
                if (depth == 0) return 0;  // a scalar body: no children; the rest is ignored
                expect_value = false;
            }
        }
        // after a value inside a container
        if (depth == 0) return count;  // the top-level container closed; the rest is ignored
        skip_ws(c);
        if (c.i >= c.n) return -1;
        const bool obj = (stk[(depth - 1) >> 5] >> ((depth - 1) & 31)) & 1u;
        const uint8_t ch = c.p[c.i];
        if (ch == ',') {
            ++c.i;
            skip_ws(c);
            if (obj) {
                if (c.i >= c.n || c.p[c.i] != '"' || !parse_string(c)) return -1;
                skip_ws(c);
                if (c.i >= c.n || c.p[c.i] != ':') return -1;
                ++c.i;
                skip_ws(c);
            }
            expect_value = true;
        } else if (ch == (obj ? '}' : ']')) {
            ++c.i;
            --depth;
            expect_value = false;
        } else {
            return -1;
        }
    }
}

// ---- flat arrays of numbers, one warp per body ------------------------------------
//
// Up to the first ']' the body must hold only whitespace (1..32), number
// characters, ',' and one '[' as its first token; anything else there (a NUL,
// a byte-order mark, a quote, a brace, a letter, a second '[') or no ']' at
// all sends the body to the general path.  Inside that form cJSON's parse is
// decided token by token: a number must follow '[' or ',', a ',' must follow
// a number, the ']' must follow a number or the '[', and a number's run of
// number characters must start with '-' or a digit and be consumed whole by
// strtod (63 characters at most).  The first event in the text decides: an
// error first is cJSON's error ("Invalid JSON"), a general-path byte first
// hands the body over.
enum : uint32_t { kTokNone = 0, kTokNum = 1, kTokComma = 2, kTokOpen = 3, kTokClose = 4 };
enum : uint32_t { kClsNum = 1, kClsComma = 2, kClsOpen = 4, kClsClose = 8, kClsBad = 16 };  // whitespace: 0
constexpr uint32_t kNoEvent = 0xFFFFFFFFu;
constexpr int kFlatWarps = 8;    // bodies per block
constexpr int kQueue = 512;      // per warp: number starts waiting for conversion (ring)

__device__ __forceinline__ uint32_t byte_class(uint32_t c) {
    if (c == 0) return kClsBad;  // a NUL ends the text: the general path
    if (c <= 32) return 0;
    if ((c >= '0' && c <= '9') || c == '+' || c == '-' || c == 'e' || c == 'E' || c == '.') return kClsNum;
    if (c == ',') return kClsComma;
    if (c == '[') return kClsOpen;
    if (c == ']') return kClsClose;
    return kClsBad;
}

// bit k of the result = bit 0 of byte k of m (k < 4)
__device__ __forceinline__ uint32_t bits4(uint32_t m) { return ((m & 0x01010101u) * 0x01020408u) >> 24; }

// One number of a flat body: checks cJSON's rules (a '-' or a digit first,
// the whole run consumed by strtod, at most 63 characters) and converts it.
__device__ __forceinline__ bool flat_number(const uint8_t* body, uint32_t len, uint32_t pos, double* v) {
    const uint8_t c0 = body[pos];
    if (!(c0 == '-' || (c0 >= '0' && c0 <= '9'))) return false;
    const int avail = len - pos < 64u ? (int)(len - pos) : 64;
    Dec d;
    int run = 0;
    const int used = scan_number(body + pos, avail, d, &run);
    if (used != run || (run == 63 && avail > 63 && is_num_char(body[pos + 63]))) return false;
    *v = to_double(d, body + pos, used);
    return true;
}

__global__ void __launch_bounds__(kFlatWarps * 32) k_decode_flat(const uint8_t* __restrict__ text,
                                                               const uint64_t* __restrict__ off, int nreq,
                                                               int64_t dim, double* __restrict__ out,
                                                               int32_t* __restrict__ status,
                                                               uint8_t* __restrict__ slow) {
    __shared__ uint8_t s_cls[256];
    __shared__ uint32_t s_queue[kFlatWarps][kQueue];
    for (int c = threadIdx.x; c < 256; c += blockDim.x) s_cls[c] = (uint8_t)byte_class((uint32_t)c);
    __syncthreads();
    const int lane = threadIdx.x & 31, wib = threadIdx.x >> 5;
    const int r = blockIdx.x * kFlatWarps + wib;
    if (r >= nreq) return;  // the whole warp
    const int64_t lo = (int64_t)off[r], hi = (int64_t)off[r + 1];
    if (hi - lo >= (1ll << 31)) {  // positions below are 32-bit
        if (lane == 0) slow[r] = 1;
        return;
    }
    const uint32_t len = (uint32_t)(hi - lo);
    const uint8_t* body = text + lo;
    double* o = out + (int64_t)r * dim;
    uint32_t* queue = s_queue[wib];
    uint32_t ev_bad = kNoEvent, ev_slow = kNoEvent;  // earliest error / general-path byte (offsets in the body)
    uint32_t carry_tok = kTokNone, carry_num = 0;    // last token before this step; last byte a number character
    uint32_t head = 0, tail = 0;                     // numbers converted / found so far (= their indexes)
    bool ended = false;
    for (int64_t base = lo & ~15ll; base < hi; base += 512) {
        const int64_t cb = base + lane * 16;
        uint4 v = make_uint4(0u, 0u, 0u, 0u);
        if (cb < hi) v = *reinterpret_cast<const uint4*>(text + cb);  // 16-aligned, inside the text buffer
        uint32_t vmask = 0xFFFFu;  // bytes of this body
        if (cb < lo) vmask &= 0xFFFFu << (uint32_t)(lo - cb);
        if (cb + 16 > hi) vmask &= cb >= hi ? 0u : (1u << (uint32_t)(hi - cb)) - 1u;
        uint32_t mnum = 0, mcom = 0, mopen = 0, mclose = 0, mbad = 0;
#pragma unroll
        for (int k = 0; k < 4; ++k) {
            const uint32_t word = k == 0 ? v.x : (k == 1 ? v.y : (k == 2 ? v.z : v.w));
            const uint32_t f = (uint32_t)s_cls[word & 0xffu] | ((uint32_t)s_cls[(word >> 8) & 0xffu] << 8) |
                               ((uint32_t)s_cls[(word >> 16) & 0xffu] << 16) | ((uint32_t)s_cls[word >> 24] << 24);
            mnum |= bits4(f) << (4 * k);
            mcom |= bits4(f >> 1) << (4 * k);
            mopen |= bits4(f >> 2) << (4 * k);
            mclose |= bits4(f >> 3) << (4 * k);
            mbad |= bits4(f >> 4) << (4 * k);
        }
        mnum &= vmask;
        mcom &= vmask;
        mopen &= vmask;
        mclose &= vmask;
        mbad &= vmask;
        // the first ']' ends the array: nothing after it counts
        const uint32_t with_close = __ballot_sync(0xffffffffu, mclose != 0);
        uint32_t mend = 0;
        if (with_close) {
            const int lc = __ffs(with_close) - 1;
            if (lane > lc) {
                mnum = mcom = mopen = mbad = 0;
            } else if (lane == lc) {
                mend = mclose & (0u - mclose);  // lowest set bit
                const uint32_t keep = mend - 1;
                mnum &= keep;
                mcom &= keep;
                mopen &= keep;
                mbad &= keep;
            }
            ended = true;
        }
        if (mbad) ev_slow = min(ev_slow, (uint32_t)(cb + __ffs(mbad) - 1 - lo));
        // number runs continuing from the previous byte are not new tokens
        uint32_t prev_num = __shfl_up_sync(0xffffffffu, (mnum >> 15) & 1u, 1);
        if (lane == 0) prev_num = carry_num;
        const uint32_t mstart = mnum & ~((mnum << 1) | prev_num);
        const uint32_t tok = mstart | mcom | mopen | mend;
        // the token before each lane's first one, and the numbers before it: warp scans
        uint32_t last = kTokNone;
        if (tok) {
            const uint32_t hb = 1u << (31 - __clz(tok));
            last = (mstart & hb) ? kTokNum : (mcom & hb) ? kTokComma : (mopen & hb) ? kTokOpen : kTokClose;
        }
        uint32_t incl = last;
        const uint32_t nnum = __popc(mstart);
        uint32_t nincl = nnum;
#pragma unroll
        for (int d = 1; d < 32; d <<= 1) {
            const uint32_t u = __shfl_up_sync(0xffffffffu, incl, d);
            const uint32_t s = __shfl_up_sync(0xffffffffu, nincl, d);
            if (lane >= d) {
                if (incl == kTokNone) incl = u;
                nincl += s;
            }
        }
        uint32_t pred = __shfl_up_sync(0xffffffffu, incl, 1);
        if (lane == 0 || pred == kTokNone) pred = carry_tok;
        uint32_t qi = tail + nincl - nnum;
        for (uint32_t t = tok; t;) {
            const int b = __ffs(t) - 1;
            t &= t - 1;
            const uint32_t bit = 1u << b;
            const uint32_t pos = (uint32_t)(cb + b - lo);
            const uint32_t ty = (mstart & bit) ? kTokNum : (mcom & bit) ? kTokComma : (mopen & bit) ? kTokOpen : kTokClose;
            if (ty == kTokNum) queue[qi++ & (kQueue - 1)] = pos;  // every number start: [head, tail) is filled
            if (ty == kTokOpen) {
                if (pred != kTokNone) ev_slow = min(ev_slow, pos);  // nested: the general path
            } else if (pred == kTokNone) {
                ev_slow = min(ev_slow, pos);  // the body does not start with '['
            } else if (ty == kTokNum) {
                if (pred != kTokOpen && pred != kTokComma) ev_bad = min(ev_bad, pos);
            } else if (ty == kTokComma) {
                if (pred != kTokNum) ev_bad = min(ev_bad, pos);
            } else if (pred == kTokComma) {
                ev_bad = min(ev_bad, pos);  // "[1,]"
            }
            pred = ty;
        }
        tail += __shfl_sync(0xffffffffu, nincl, 31);
        const uint32_t lt = __shfl_sync(0xffffffffu, incl, 31);
        if (lt != kTokNone) carry_tok = lt;
        carry_num = __shfl_sync(0xffffffffu, (mnum >> 15) & 1u, 31);
        const bool stop = __any_sync(0xffffffffu, ev_bad != kNoEvent || ev_slow != kNoEvent) || ended;
        __syncwarp();
        // convert 32 numbers at a time, one per lane (all of them before leaving)
        while (tail - head >= 32u || (stop && tail != head)) {
            const uint32_t i = head + lane;
            if (i < tail) {
                const uint32_t pos = queue[i & (kQueue - 1)];
                double x;
                if (!flat_number(body, len, pos, &x))
                    ev_bad = min(ev_bad, pos);
                else if (i < (uint64_t)dim)
                    o[i] = x;
            }
            head = tail - head >= 32u ? head + 32u : tail;
        }
        __syncwarp();
        if (stop) break;
    }
    if (!ended) ev_slow = min(ev_slow, len);  // no ']': the general path decides
    ev_bad = __reduce_min_sync(0xffffffffu, ev_bad);
    ev_slow = __reduce_min_sync(0xffffffffu, ev_slow);
    __syncwarp();  // the lanes' value stores come before the fill below
    if (ev_slow < ev_bad) {
        if (lane == 0) slow[r] = 1;
        return;
    }
    int32_t st = SVDB_DEC_OK;
    if (ev_bad != kNoEvent)
        st = SVDB_DEC_INVALID_JSON;
    else if ((int64_t)tail != dim)
        st = SVDB_DEC_SIZE_MISMATCH;
    if (st != SVDB_DEC_OK)
        for (int64_t k = lane; k < dim; k += 32) o[k] = __longlong_as_double(0x7ff8000000000000ll);
    if (lane == 0) {
        status[r] = st;
        slow[r] = 0;
    }
}

// ---- the general path ---------------------------------------------------------------
__global__ void k_decode_parse(const uint8_t* __restrict__ text, const uint64_t* __restrict__ off, int nreq,
                               int64_t dim, const uint8_t* __restrict__ slow, int64_t* __restrict__ child,
                               int32_t* __restrict__ status) {
    const int r = blockIdx.x * blockDim.x + threadIdx.x;
    if (r >= nreq || !slow[r]) return;
    const int64_t lo = (int64_t)off[r], hi = (int64_t)off[r + 1];
    const int64_t cnt = parse_body(text + lo, hi - lo, child + (int64_t)r * dim, dim);
    int32_t st = SVDB_DEC_OK;
    if (cnt < 0)
        st = SVDB_DEC_INVALID_JSON;
    else if (cnt != dim)
        st = SVDB_DEC_SIZE_MISMATCH;
    else
        for (int64_t k = 0; k < dim; ++k)
            if (child[(int64_t)r * dim + k] < 0) {
                st = SVDB_DEC_INVALID_DATA;
                break;
            }
    status[r] = st;
}

__global__ void k_decode_numbers(const uint8_t* __restrict__ text, const uint64_t* __restrict__ off, int nreq,
                                 int64_t dim, const uint8_t* __restrict__ slow, const int64_t* __restrict__ child,
                                 const int32_t* __restrict__ status, double* __restrict__ out) {
    const int64_t r = blockIdx.x;  // one block per body; bodies the flat decoder finished leave at once
    if (r >= nreq || !slow[r]) return;
    const bool ok = status[r] == SVDB_DEC_OK;
    const int64_t lo = (int64_t)off[r], hi = (int64_t)off[r + 1];
    for (int64_t t = r * dim + threadIdx.x; t < (r + 1) * dim; t += blockDim.x) {
        if (!ok) {
            out[t] = __longlong_as_double(0x7ff8000000000000ll);
            continue;
        }
        const int64_t at = lo + child[t];
        Dec d;
        const int used = scan_number(text + at, hi - at < 64 ? (int)(hi - at) : 64, d);
        out[t] = to_double(d, text + at, used);
    }
}

bool host_pinned(const void* p) {
    if (!p) return false;
    cudaPointerAttributes at;
    if (cudaPointerGetAttributes(&at, p) != cudaSuccess) {
        cudaGetLastError();
        return false;
    }
    return at.type == cudaMemoryTypeHost;
}

// ---------------------------------------------------------------------------
// Response bodies as cJSON_PrintUnformatted writes them.
//
// The handlers build their answers with cJSON and print them unformatted
// (src/compare_handler.c:180-185 for /compare, :409-424 for /nearest).
// cJSON's number rule (published 1.7 sources, restated): "null" for NaN or an
// infinity; the decimal integer when the value equals its int conversion
// (clamped to INT_MIN..INT_MAX; -0 prints "0"); otherwise the text of
// printf's "%1.15g" if strtod of it lies within DBL_EPSILON (relative to the
// larger magnitude) of the value, else "%1.17g".  printf's %g is exact: the
// value's decimal expansion rounded to the precision, half to even on an
// exact tie.  Here the first 18 significant digits and a sticky bit come from
// exact big-integer arithmetic (m 2^e, or m 5^-e 10^e for e < 0, divided by
// powers of ten), the round trip uses the decoder's own exact conversion, and
// the text follows %g's layout (fixed when -4 <= X < P, else d.ddde+XX,
// trailing zeros and a bare point dropped).
// ---------------------------------------------------------------------------
constexpr int kFmtLimbs = 82;  // 2624 bits >= bits(2^53 x 5^1074) (2547)
struct B32 {
    uint32_t v[kFmtLimbs];
    int n;
};

__device__ __forceinline__ void b32_mul(B32& b, uint32_t m) {
    uint64_t c = 0;
    for (int i = 0; i < b.n; ++i) {
        const uint64_t t = (uint64_t)b.v[i] * m + c;
        b.v[i] = (uint32_t)t;
        c = t >> 32;
    }
    if (c && b.n < kFmtLimbs) b.v[b.n++] = (uint32_t)c;
}
// b /= d, returns the remainder
__device__ __forceinline__ uint32_t b32_divrem(B32& b, uint32_t d) {
    uint64_t r = 0;
    for (int i = b.n - 1; i >= 0; --i) {
        const uint64_t cur = (r << 32) | b.v[i];
        b.v[i] = (uint32_t)(cur / d);
        r = cur % d;
    }
    while (b.n > 0 && b.v[b.n - 1] == 0) --b.n;
    return (uint32_t)r;
}
__device__ __forceinline__ uint32_t b32_divrem_1e9(B32& b) {  // constant divisor: multiply-high code
    uint64_t r = 0;
    for (int i = b.n - 1; i >= 0; --i) {
        const uint64_t cur = (r << 32) | b.v[i];
        b.v[i] = (uint32_t)(cur / 1000000000ull);
        r = cur % 1000000000ull;
    }
    while (b.n > 0 && b.v[b.n - 1] == 0) --b.n;
    return (uint32_t)r;
}
__device__ __forceinline__ int b32_bits(const B32& b) {
    return b.n ? 32 * (b.n - 1) + (32 - __clz((int)b.v[b.n - 1])) : 0;
}

__device__ __constant__ uint64_t c_pow10[20] = {1ull,
                                                10ull,
                                                100ull,
                                                1000ull,
                                                10000ull,
                                                100000ull,
                                                1000000ull,
                                                10000000ull,
                                                100000000ull,
                                                1000000000ull,
                                                10000000000ull,
                                                100000000000ull,
                                                1000000000000ull,
                                                10000000000000ull,
                                                100000000000000ull,
                                                1000000000000000ull,
                                                10000000000000000ull,
                                                100000000000000000ull,
                                                1000000000000000000ull,
                                                10000000000000000000ull};

__device__ __forceinline__ int u64_digits(uint64_t x) {  // decimal digits of x > 0
    int L = 1;
    while (L < 20 && x >= c_pow10[L]) ++L;
    return L;
}

// The exact value m 2^e (m > 0): its first 18 significant digits D
// (10^17 <= D < 10^18), whether any later digit is nonzero, and the decimal
// exponent of its first digit.
__device__ void exact_digits18(uint64_t m, int e, uint64_t* D, bool* sticky, int* E10) {
    B32 N;
    N.v[0] = (uint32_t)m;
    N.v[1] = (uint32_t)(m >> 32);
    N.n = N.v[1] ? 2 : 1;
    int k10 = 0;  // value = N x 10^k10
    if (e >= 0) {
        const int w = e >> 5, bsh = e & 31;
        for (int i = N.n - 1; i >= 0; --i) N.v[i + w] = N.v[i];
        for (int i = 0; i < w; ++i) N.v[i] = 0;
        N.n += w;
        if (bsh) {
            uint32_t carry = 0;
            for (int i = 0; i < N.n; ++i) {
                const uint32_t x = N.v[i];
                N.v[i] = (x << bsh) | carry;
                carry = x >> (32 - bsh);
            }
            if (carry) N.v[N.n++] = carry;
        }
    } else {  // m 2^e = m 5^-e 10^e
        int k = -e;
        while (k >= 13) {
            b32_mul(N, 1220703125u);  // 5^13
            k -= 13;
        }
        uint32_t r = 1;
        while (k-- > 0) r *= 5;
        if (r > 1) b32_mul(N, r);
        k10 = e;
    }
    bool st = false;
    int L;
    uint64_t x;
    const int bits = b32_bits(N);
    if (bits <= 64) {
        x = N.n == 1 ? N.v[0] : ((uint64_t)N.v[1] << 32) | N.v[0];
        L = u64_digits(x);
        if (L <= 18) {
            x *= c_pow10[18 - L];
        } else {
            const uint64_t p = c_pow10[L - 18];
            st = x % p != 0;
            x /= p;
        }
    } else {
        // digits of N: L in {Lg, Lg + 1}, Lg = floor((bits - 1) log10 2) + 1 (a
        // lower bound; the margin keeps the floor from rounding up)
        const int Lg = (int)floor((double)(bits - 1) * 0.30102999566398119521 - 1e-9) + 1;
        int sdrop = Lg - 18;  // >= 2: bits > 64 means Lg >= 20
        while (sdrop >= 9) {
            st |= b32_divrem_1e9(N) != 0;
            sdrop -= 9;
        }
        if (sdrop > 0) st |= b32_divrem(N, (uint32_t)c_pow10[sdrop]) != 0;
        x = N.n == 0 ? 0 : N.n == 1 ? N.v[0] : ((uint64_t)N.v[1] << 32) | N.v[0];  // < 10^19
        L = Lg;
        if (x >= c_pow10[18]) {
            st |= x % 10 != 0;
            x /= 10;
            L = Lg + 1;
        }
    }
    *D = x;
    *sticky = st;
    *E10 = L - 1 + k10;
}

// D18 rounded to P significant digits, half to even: q (10^(P-1) <= q < 10^P)
// and the decimal exponent X of its first digit
__device__ __forceinline__ void round_digits(uint64_t D18, bool sticky, int E10, int P, uint64_t* q, int* X) {
    const uint64_t div = c_pow10[18 - P], half = div / 2;
    uint64_t t = D18 / div;
    const uint64_t r = D18 % div;
    if (r > half || (r == half && (sticky || (t & 1)))) ++t;
    int x = E10;
    if (t == c_pow10[P]) {
        t = c_pow10[P - 1];
        ++x;
    }
    *q = t;
    *X = x;
}

// printf %.<P>g of the value sign q 10^(X - P + 1)
__device__ int g_text(bool neg, uint64_t q, int X, int P, char* out) {
    char dg[20];
    for (int i = P - 1; i >= 0; --i) {
        dg[i] = (char)('0' + q % 10);
        q /= 10;
    }
    int nd = P;
    while (nd > 1 && dg[nd - 1] == '0') --nd;
    int o = 0;
    if (neg) out[o++] = '-';
    if (X < -4 || X >= P) {
        out[o++] = dg[0];
        if (nd > 1) {
            out[o++] = '.';
            for (int i = 1; i < nd; ++i) out[o++] = dg[i];
        }
        out[o++] = 'e';
        out[o++] = X < 0 ? '-' : '+';
        const int ax = X < 0 ? -X : X;
        if (ax >= 100) out[o++] = (char)('0' + ax / 100);
        out[o++] = (char)('0' + (ax / 10) % 10);
        out[o++] = (char)('0' + ax % 10);
    } else if (X >= 0) {
        for (int i = 0; i <= X; ++i) out[o++] = dg[i];
        if (nd > X + 1) {
            out[o++] = '.';
            for (int i = X + 1; i < nd; ++i) out[o++] = dg[i];
        }
    } else {
        out[o++] = '0';
        out[o++] = '.';
        for (int i = 0; i < -X - 1; ++i) out[o++] = '0';
        for (int i = 0; i < nd; ++i) out[o++] = dg[i];
    }
    return o;
}

__device__ int int_text(int v, char* out) {
    char t[12];
    int n = 0, o = 0;
    uint32_t u = v < 0 ? (uint32_t)(-(int64_t)v) : (uint32_t)v;
    do {
        t[n++] = (char)('0' + u % 10);
        u /= 10;
    } while (u);
    if (v < 0) out[o++] = '-';
    while (n) out[o++] = t[--n];
    return o;
}

// one number as cJSON prints it; at most 24 bytes
__device__ int cjson_number(double d, char* out) {
    if (isnan(d) || isinf(d)) {
        out[0] = 'n';
        out[1] = 'u';
        out[2] = 'l';
        out[3] = 'l';
        return 4;
    }
    const int vi = d >= 2147483647.0 ? 2147483647 : d <= -2147483648.0 ? (-2147483647 - 1) : (int)d;
    if (d == (double)vi) return int_text(vi, out);
    const uint64_t b = (uint64_t)__double_as_longlong(d);
    const bool neg = (b >> 63) != 0;
    const int be = (int)((b >> 52) & 0x7ff);
    uint64_t m = b & ((1ull << 52) - 1);
    int e;
    if (be == 0) {
        e = -1074;
    } else {
        m |= 1ull << 52;
        e = be - 1075;
    }
    uint64_t D18;
    bool sticky;
    int E10;
    exact_digits18(m, e, &D18, &sticky, &E10);
    uint64_t q;
    int X;
    round_digits(D18, sticky, E10, 15, &q, &X);
    // strtod of the 15-digit text is the correctly rounded q 10^(X - 14)
    const double back = value_of(q, (int64_t)X - 14, neg);
    const double mx = fmax(fabs(back), fabs(d));
    if (__dsub_rn(fmax(back, d), fmin(back, d)) <= __dmul_rn(mx, 2.220446049250313e-16))
        return g_text(neg, q, X, 15, out);
    round_digits(D18, sticky, E10, 17, &q, &X);
    return g_text(neg, q, X, 17, out);
}

// a C string (at most maxlen bytes, up to its NUL) as cJSON quotes it
__device__ int cjson_string(const char* s, int maxlen, char* out) {
    int o = 0;
    out[o++] = '"';
    for (int i = 0; i < maxlen && s[i]; ++i) {
        const unsigned char c = (unsigned char)s[i];
        if (c == '"' || c == '\\') {
            out[o++] = '\\';
            out[o++] = (char)c;
        } else if (c < 32) {
            out[o++] = '\\';
            if (c == '\b') out[o++] = 'b';
            else if (c == '\f') out[o++] = 'f';
            else if (c == '\n') out[o++] = 'n';
            else if (c == '\r') out[o++] = 'r';
            else if (c == '\t') out[o++] = 't';
            else {
                const char* hx = "0123456789abcdef";
                out[o++] = 'u';
                out[o++] = '0';
                out[o++] = '0';
                out[o++] = hx[c >> 4];
                out[o++] = hx[c & 15];
            }
        } else {
            out[o++] = (char)c;
        }
    }
    out[o++] = '"';
    return o;
}

__device__ __forceinline__ int put_lit(char* out, const char* lit) {
    int o = 0;
    while (lit[o]) {
        out[o] = lit[o];
        ++o;
    }
    return o;
}

// GET /compare answers, one thread each, into slots of kCmpSlot bytes
constexpr int kCmpSlot = 64;
__global__ void k_fmt_compare(const int32_t* __restrict__ metric, const float* __restrict__ value,
                              const int32_t* __restrict__ status, int n, char* __restrict__ slots,
                              uint32_t* __restrict__ len) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    char* o = slots + (size_t)i * kCmpSlot;
    int k = 0;
    const int st = status[i];
    if (st == 0) {
        const int m = metric[i];
        k += put_lit(o, m == 0 ? "{\"cosine_similarity\":" : m == 1 ? "{\"euclidean_distance\":" : "{\"dot_product\":");
        k += cjson_number((double)value[i], o + k);
        o[k++] = '}';
    } else {  // the handler's fixed error bodies (src/compare_handler.c:103-163)
        k += put_lit(o, st == 1   ? "{\"error\": \"Index out of bounds\"}"
                        : st == 2 ? "{\"error\": \"Vector not found\"}"
                        : st == 3 ? "{\"error\": \"Vectors have different dimensions\"}"
                        : st == 4 ? "{\"error\": \"Vector size mismatch\"}"
                                  : "{\"error\": \"Unknown comparison method\"}");
    }
    len[i] = (uint32_t)k;
}

// POST /nearest answers, one block each, into slots of `slot` bytes: the row's
// numbers are printed by all threads into shared memory (kNumSlot bytes each),
// in chunks, and placed by a block scan of their lengths
constexpr int kFmtThreads = 256;
constexpr int kNumSlot = 26;       // a number (<= 24 bytes) and its comma
constexpr int kFmtChunk = 1024;    // numbers per shared-memory pass
__global__ void __launch_bounds__(kFmtThreads) k_fmt_nearest(const int32_t* __restrict__ kind,
                                                             const uint64_t* __restrict__ index,
                                                             const double* const* __restrict__ rows,
                                                             const uint32_t* __restrict__ dims,
                                                             const char* __restrict__ uuids, size_t slot,
                                                             char* __restrict__ slots, uint32_t* __restrict__ len) {
    __shared__ char buf[kFmtChunk * kNumSlot];
    __shared__ uint32_t pos[kFmtChunk];
    __shared__ uint8_t lens[kFmtChunk];
    __shared__ uint32_t wsum[kFmtThreads / 32];
    __shared__ uint32_t s_at;
    const int r = blockIdx.x;
    char* o = slots + (size_t)r * slot;
    const int kd = kind[r];
    if (kd <= 0) {
        if (threadIdx.x == 0)
            len[r] = (uint32_t)put_lit(o, kd == 0 ? "{\"error\":\"No nearest neighbor found\"}"
                                                  : "{\"error\":\"Nearest neighbor not found\"}");
        return;
    }
    if (threadIdx.x == 0) {
        int k = put_lit(o, "{\"index\":");
        k += cjson_number((double)index[r], o + k);
        k += put_lit(o + k, ",\"vector\":[");
        s_at = (uint32_t)k;
    }
    __syncthreads();
    const double* row = rows[r];
    const int d = (int)dims[r];
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    constexpr int per = kFmtChunk / kFmtThreads;  // numbers per thread and chunk, contiguous
    for (int c0 = 0; c0 < d; c0 += kFmtChunk) {
        const int cn = min(kFmtChunk, d - c0);
        uint32_t tot = 0;
#pragma unroll
        for (int u = 0; u < per; ++u) {
            const int j = threadIdx.x * per + u;
            if (j < cn) {
                char* b = buf + j * kNumSlot;
                int k = 0;
                if (c0 + j) b[k++] = ',';
                k += cjson_number(row[c0 + j], b + k);
                lens[j] = (uint8_t)k;
                tot += (uint32_t)k;
            }
        }
        // exclusive scan of the threads' totals: each thread's numbers in order
        uint32_t incl = tot;
        for (int sh = 1; sh < 32; sh <<= 1) {
            const uint32_t t = __shfl_up_sync(0xffffffffu, incl, sh);
            if (lane >= sh) incl += t;
        }
        if (lane == 31) wsum[warp] = incl;
        __syncthreads();
        uint32_t wbase = 0, total = 0;
        for (int w = 0; w < kFmtThreads / 32; ++w) {
            if (w < warp) wbase += wsum[w];
            total += wsum[w];
        }
        uint32_t at = s_at + wbase + incl - tot;
#pragma unroll
        for (int u = 0; u < per; ++u) {
            const int j = threadIdx.x * per + u;
            if (j < cn) {
                pos[j] = at;
                at += lens[j];
            }
        }
        __syncthreads();
        for (int j = warp; j < cn; j += kFmtThreads / 32)  // a number is at most 25 bytes: a warp copies it
            if (lane < (int)lens[j]) o[pos[j] + lane] = buf[j * kNumSlot + lane];
        __syncthreads();
        if (threadIdx.x == 0) s_at += total;
        __syncthreads();
    }
    if (threadIdx.x == 0) {
        int k = (int)s_at;
        k += put_lit(o + k, "],\"uuid\":");
        k += cjson_string(uuids + (size_t)r * 37, 37, o + k);
        o[k++] = '}';
        len[r] = (uint32_t)k;
    }
}

// slots -> one packed text at the given offsets
__global__ void k_fmt_pack(const char* __restrict__ slots, size_t slot, const uint32_t* __restrict__ len,
                           const uint64_t* __restrict__ off, int n, char* __restrict__ out) {
    const int r = blockIdx.x;
    if (r >= n) return;
    const char* src = slots + (size_t)r * slot;
    char* dst = out + off[r];
    for (uint32_t t = threadIdx.x; t < len[r]; t += blockDim.x) dst[t] = src[t];
}

}  // namespace

// Decode n bodies (host bytes text[off[i] .. off[i+1])) into n x dim doubles.
// Page-locked text and outputs are read and written by DMA directly; pageable
// ones go through the context's staging buffer.  Large batches are taken in
// up to kChunks chunks on kStreams streams, so one chunk's copy to the device
// overlaps another's kernels and copy back.  A chunk keeps at least 2,048
// bodies (256 blocks of the one-warp-per-body decoder): at 4,096 bodies of
// 768 numbers, 2 chunks take 0.70 ms against 0.81 ms for one, and 8 chunks
// of 512 bodies (64 blocks each) 0.98 ms.
constexpr int kStreams = 3, kChunks = 4;
constexpr size_t kChunkBodies = 2048, kChunkText = 4u << 20;

int decode_bodies(Store* s, const char* text, const uint64_t* off, size_t n, size_t dim, double* out,
                  int32_t* status) {
    if (n == 0) return SVDB_OK;
    const size_t tb = off[n] - off[0];
    const size_t ob = (n + 1) * sizeof(uint64_t);
    const size_t cb = n * dim * sizeof(int64_t), vb = n * dim * sizeof(double), sb = n * sizeof(int32_t);
    const size_t a_text = round_up(tb + 1, 256), a_off = round_up(ob, 256), a_ch = round_up(cb, 256),
                 a_val = round_up(vb, 256), a_st = round_up(sb, 256);
    int rc = s->scratch_reserve(a_text + a_off + a_ch + a_val + a_st + n + 256);
    if (!rc) rc = s->pinned_reserve(std::max(round_up(tb, 8) + ob, vb + sb));
    if (rc) return rc;
    uint8_t* base = (uint8_t*)s->scratch;
    uint8_t* dtext = base;
    uint64_t* doff = (uint64_t*)(base + a_text);
    int64_t* dch = (int64_t*)(base + a_text + a_off);
    double* dval = (double*)(base + a_text + a_off + a_ch);
    int32_t* dst = (int32_t*)(base + a_text + a_off + a_ch + a_val);
    uint8_t* dslow = base + a_text + a_off + a_ch + a_val + a_st;
    uint8_t* hp = (uint8_t*)s->pin;
    // per process (one context); callers hold the decode mutex
    static bool ready = false;
    static cudaStream_t streams[kStreams];
    static cudaEvent_t ev_ready, ev_done[kStreams];
    if (!ready) {
        for (int i = 0; i < kStreams; ++i) {
            SVDB_CUDA(cudaStreamCreateWithFlags(&streams[i], cudaStreamNonBlocking));
            SVDB_CUDA(cudaEventCreateWithFlags(&ev_done[i], cudaEventDisableTiming));
        }
        SVDB_CUDA(cudaEventCreateWithFlags(&ev_ready, cudaEventDisableTiming));
        k_pow5_init<<<(kP5Max - kP5Min + 128) / 128, 128, 0, s->stream>>>();
        SVDB_LAUNCH_CHECK();
        ready = true;
    }
    const bool pin_in = host_pinned(text + off[0]);
    const bool pin_out = host_pinned(out) && host_pinned(status);
    if (!pin_in) std::memcpy(hp, text + off[0], tb);
    uint64_t* hoff = (uint64_t*)(hp + round_up(tb, 8));
    for (size_t i = 0; i <= n; ++i) hoff[i] = off[i] - off[0];
    SVDB_CUDA(cudaMemcpyAsync(doff, hoff, ob, cudaMemcpyHostToDevice, s->stream));
    SVDB_CUDA(cudaEventRecord(ev_ready, s->stream));
    const size_t nch =
        std::max<size_t>(1, std::min(std::min((size_t)kChunks, n / kChunkBodies), tb / kChunkText));
    for (size_t c = 0; c < nch; ++c) {
        cudaStream_t st = streams[c % kStreams];
        const size_t b0 = c * n / nch, b1 = (c + 1) * n / nch, m = b1 - b0;
        const size_t t0 = off[b0] - off[0], t1 = off[b1] - off[0];
        SVDB_CUDA(cudaStreamWaitEvent(st, ev_ready, 0));
        SVDB_CUDA(cudaMemcpyAsync(dtext + t0, pin_in ? (const void*)(text + off[b0]) : (const void*)(hp + t0), t1 - t0,
                                  cudaMemcpyHostToDevice, st));
        k_decode_flat<<<(unsigned)((m + kFlatWarps - 1) / kFlatWarps), kFlatWarps * 32, 0, st>>>(
            dtext, doff + b0, (int)m, (int64_t)dim, dval + b0 * dim, dst + b0, dslow + b0);
        SVDB_LAUNCH_CHECK();
        k_decode_parse<<<(unsigned)((m + 63) / 64), 64, 0, st>>>(dtext, doff + b0, (int)m, (int64_t)dim, dslow + b0,
                                                                 dch + b0 * dim, dst + b0);
        SVDB_LAUNCH_CHECK();
        if (dim) {
            k_decode_numbers<<<(unsigned)m, 128, 0, st>>>(dtext, doff + b0, (int)m, (int64_t)dim, dslow + b0,
                                                          dch + b0 * dim, dst + b0, dval + b0 * dim);
            SVDB_LAUNCH_CHECK();
        }
        if (pin_out) {
            SVDB_CUDA(cudaMemcpyAsync(out + b0 * dim, dval + b0 * dim, m * dim * sizeof(double),
                                      cudaMemcpyDeviceToHost, st));
            SVDB_CUDA(cudaMemcpyAsync(status + b0, dst + b0, m * sizeof(int32_t), cudaMemcpyDeviceToHost, st));
        }
    }
    for (size_t i = 0; i < std::min<size_t>(nch, kStreams); ++i) {
        SVDB_CUDA(cudaEventRecord(ev_done[i], streams[i]));
        SVDB_CUDA(cudaStreamWaitEvent(s->stream, ev_done[i], 0));
    }
    SVDB_CUDA(cudaStreamSynchronize(s->stream));
    if (pin_out) return SVDB_OK;
    // the staging buffer held the text; now it takes the results
    SVDB_CUDA(cudaMemcpyAsync(hp, dval, vb, cudaMemcpyDeviceToHost, s->stream));
    SVDB_CUDA(cudaMemcpyAsync(hp + vb, dst, sb, cudaMemcpyDeviceToHost, s->stream));
    SVDB_CUDA(cudaStreamSynchronize(s->stream));
    std::memcpy(out, hp, vb);
    std::memcpy(status, hp + vb, sb);
    return SVDB_OK;
}

// ---- response bodies: host side ---------------------------------------------
// The power-of-five table of the exact conversion (the formatter's round-trip
// check uses it), once per process, finished before any formatter runs.
static int ensure_pow5(cudaStream_t st) {
    static std::mutex mu;
    static bool done = false;
    std::lock_guard<std::mutex> lk(mu);
    if (done) return SVDB_OK;
    k_pow5_init<<<(kP5Max - kP5Min + 128) / 128, 128, 0, st>>>();
    SVDB_LAUNCH_CHECK();
    SVDB_CUDA(cudaStreamSynchronize(st));
    done = true;
    return SVDB_OK;
}

// lengths -> offsets on the host; then, when `out` has room, the slots packed
// on the device and copied out as one text
static int fmt_finish(Store* s, size_t n, const char* d_slots, size_t slot, const uint32_t* d_len, uint64_t* d_off,
                      char* d_packed, char* out, size_t cap, uint64_t* offsets) {
    std::vector<uint32_t> hl(n);
    SVDB_CUDA(cudaMemcpyAsync(hl.data(), d_len, n * sizeof(uint32_t), cudaMemcpyDeviceToHost, s->stream));
    SVDB_CUDA(cudaStreamSynchronize(s->stream));
    offsets[0] = 0;
    for (size_t i = 0; i < n; ++i) offsets[i + 1] = offsets[i] + hl[i];
    const uint64_t total = offsets[n];
    if (!out) return SVDB_OK;  // sizes only
    if (total > cap) {
        svdb_set_error("format: the responses need %llu bytes, the buffer holds %zu", (unsigned long long)total, cap);
        return SVDB_EINVAL;
    }
    SVDB_CUDA(cudaMemcpyAsync(d_off, offsets, (n + 1) * sizeof(uint64_t), cudaMemcpyHostToDevice, s->stream));
    k_fmt_pack<<<(unsigned)n, 128, 0, s->stream>>>(d_slots, slot, d_len, d_off, (int)n, d_packed);
    SVDB_LAUNCH_CHECK();
    SVDB_CUDA(cudaMemcpyAsync(out, d_packed, total, cudaMemcpyDeviceToHost, s->stream));
    SVDB_CUDA(cudaStreamSynchronize(s->stream));
    return SVDB_OK;
}

int format_compare(Store* s, const int32_t* metric, const float* value, const int32_t* status, size_t n, char* out,
                   size_t cap, uint64_t* offsets) {
    if (n == 0) {
        offsets[0] = 0;
        return SVDB_OK;
    }
    int rc = ensure_pow5(s->stream);
    if (rc) return rc;
    const size_t a_in = round_up(n * 12, 256), a_slots = round_up(n * kCmpSlot, 256), a_len = round_up(n * 4, 256),
                 a_off = round_up((n + 1) * 8, 256);
    rc = s->scratch_reserve(a_in + 2 * a_slots + a_len + a_off);
    if (rc) return rc;
    uint8_t* base = (uint8_t*)s->scratch;
    int32_t* dm = (int32_t*)base;
    float* dv = (float*)(dm + n);
    int32_t* ds = (int32_t*)(dv + n);
    char* slots = (char*)(base + a_in);
    uint32_t* dl = (uint32_t*)(base + a_in + a_slots);
    uint64_t* doff = (uint64_t*)(base + a_in + a_slots + a_len);
    char* packed = (char*)(base + a_in + a_slots + a_len + a_off);
    SVDB_CUDA(cudaMemcpyAsync(dm, metric, n * 4, cudaMemcpyHostToDevice, s->stream));
    SVDB_CUDA(cudaMemcpyAsync(dv, value, n * 4, cudaMemcpyHostToDevice, s->stream));
    SVDB_CUDA(cudaMemcpyAsync(ds, status, n * 4, cudaMemcpyHostToDevice, s->stream));
    k_fmt_compare<<<(unsigned)((n + 127) / 128), 128, 0, s->stream>>>(dm, dv, ds, (int)n, slots, dl);
    SVDB_LAUNCH_CHECK();
    return fmt_finish(s, n, slots, kCmpSlot, dl, doff, packed, out, cap, offsets);
}

// kind[i]: 1 a row (slot[i] >= 0: the store's row; else host_rows[i]), 0 no
// neighbour, -1 an index that reads no row; dims[i] the row's dimension
int format_nearest(Store* s, size_t n, const int32_t* kind, const uint64_t* index, const int64_t* slot,
                   const uint32_t* dims, const double* const* host_rows, const char* uuids37, char* out, size_t cap,
                   uint64_t* offsets) {
    if (n == 0) {
        offsets[0] = 0;
        return SVDB_OK;
    }
    int rc = s->sync();  // staged rows onto the device
    if (!rc) rc = ensure_pow5(s->stream);
    if (rc) return rc;
    uint32_t dmax = 0;
    size_t host_doubles = 0;
    for (size_t i = 0; i < n; ++i) {
        if (kind[i] != 1) continue;
        dmax = std::max(dmax, dims[i]);
        if (slot[i] < 0) host_doubles += dims[i];
    }
    const size_t slot_bytes = round_up(64 + (size_t)kNumSlot * dmax + 6 * 37 + 64, 16);
    const size_t a_meta = round_up(n * (4 + 8 + 8 + 4 + 37), 256), a_host = round_up(host_doubles * 8, 256),
                 a_slots = round_up(n * slot_bytes, 256), a_len = round_up(n * 4, 256),
                 a_off = round_up((n + 1) * 8, 256);
    rc = s->scratch_reserve(a_meta + a_host + 2 * a_slots + a_len + a_off);
    if (rc) return rc;
    uint8_t* base = (uint8_t*)s->scratch;
    // meta block: the 8-byte fields first, so every field is aligned for any n
    std::vector<uint8_t> hm(a_meta);
    uint64_t* hi = (uint64_t*)hm.data();
    const double** hr = (const double**)(hi + n);
    int32_t* hk = (int32_t*)(hr + n);
    uint32_t* hd = (uint32_t*)(hk + n);
    char* hu = (char*)(hd + n);
    std::vector<double> hrows(host_doubles);
    double* dhost = (double*)(base + a_meta);
    size_t at = 0;
    for (size_t i = 0; i < n; ++i) {
        hk[i] = kind[i];
        hi[i] = index[i];
        hd[i] = kind[i] == 1 ? dims[i] : 0;
        hr[i] = nullptr;
        std::memcpy(hu + i * 37, uuids37 + i * 37, 37);
        if (kind[i] != 1) continue;
        if (slot[i] >= 0) {
            hr[i] = s->x64 + (size_t)slot[i] * s->ld;
        } else {
            if (dims[i]) std::memcpy(hrows.data() + at, host_rows[i], dims[i] * sizeof(double));
            hr[i] = dhost + at;
            at += dims[i];
        }
    }
    SVDB_CUDA(cudaMemcpyAsync(base, hm.data(), a_meta, cudaMemcpyHostToDevice, s->stream));
    if (host_doubles)
        SVDB_CUDA(cudaMemcpyAsync(dhost, hrows.data(), host_doubles * 8, cudaMemcpyHostToDevice, s->stream));
    const uint64_t* di = (const uint64_t*)base;
    const double* const* drows = (const double* const*)(di + n);
    const int32_t* dk = (const int32_t*)(drows + n);
    const uint32_t* ddim = (const uint32_t*)(dk + n);
    const char* du = (const char*)(ddim + n);
    char* slots = (char*)(base + a_meta + a_host);
    uint32_t* dl = (uint32_t*)(base + a_meta + a_host + a_slots);
    uint64_t* doff = (uint64_t*)(base + a_meta + a_host + a_slots + a_len);
    char* packed = (char*)(base + a_meta + a_host + a_slots + a_len + a_off);
    k_fmt_nearest<<<(unsigned)n, kFmtThreads, 0, s->stream>>>(dk, di, drows, ddim, du, slot_bytes, slots, dl);
    SVDB_LAUNCH_CHECK();
    rc = fmt_finish(s, n, slots, slot_bytes, dl, doff, packed, out, cap, offsets);
    SVDB_CUDA(cudaStreamSynchronize(s->stream));  // the host staging above is freed on return
    return rc;
}

}  // namespace svdb

// One decode context per process (stream, scratch, staging), shared by the
// callers under a mutex: decoding needs no store.
namespace {
std::mutex g_dec_mu;
svdb::Store* g_dec = nullptr;
}  // namespace

extern "C" int svdbd_decode_bodies(const char* text, const uint64_t* off, size_t n, size_t dim, double* out,
                                   int32_t* status) {
    std::lock_guard<std::mutex> lk(g_dec_mu);
    if (!g_dec) {
        g_dec = new (std::nothrow) svdb::Store();
        if (!g_dec) {
            svdb_set_error("decode: out of host memory");
            return SVDB_ENOMEM;
        }
        g_dec->dim = g_dec->ld = g_dec->ldb = 1;
    }
    int rc = g_dec->ensure();
    return rc ? rc : svdb::decode_bodies(g_dec, text, off, n, dim, out, status);
}

extern "C" int svdbd_format_compare(const int32_t* metric, const float* value, const int32_t* status, size_t n,
                                    char* out, size_t cap, uint64_t* offsets) {
    std::lock_guard<std::mutex> lk(g_dec_mu);
    if (!g_dec) {
        g_dec = new (std::nothrow) svdb::Store();
        if (!g_dec) {
            svdb_set_error("format: out of host memory");
            return SVDB_ENOMEM;
        }
        g_dec->dim = g_dec->ld = g_dec->ldb = 1;
    }
    int rc = g_dec->ensure();
    return rc ? rc : svdb::format_compare(g_dec, metric, value, status, n, out, cap, offsets);
}

extern "C" int svdbd_format_nearest(svdbd_store* hs, size_t n, const int32_t* kind, const uint64_t* index,
                                    const int64_t* slot, const uint32_t* dims, const double* const* host_rows,
                                    const char* uuids37, char* out, size_t cap, uint64_t* offsets) {
    if (hs) {
        return svdb::format_nearest(reinterpret_cast<svdb::Store*>(hs), n, kind, index, slot, dims, host_rows,
                                    uuids37, out, cap, offsets);
    }
    std::lock_guard<std::mutex> lk(g_dec_mu);  // a store with no device rows: the decode context
    if (!g_dec) {
        g_dec = new (std::nothrow) svdb::Store();
        if (!g_dec) {
            svdb_set_error("format: out of host memory");
            return SVDB_ENOMEM;
        }
        g_dec->dim = g_dec->ld = g_dec->ldb = 1;
    }
    int rc = g_dec->ensure();
    return rc ? rc : svdb::format_nearest(g_dec, n, kind, index, slot, dims, host_rows, uuids37, out, cap, offsets);
}
