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
// One thread per body validates the whole JSON text with cJSON's grammar
// (whitespace = any byte <= 32; a UTF-8 byte-order mark is skipped; nesting
// up to 1000; strings with cJSON's escape rules; literals null / true /
// false; content after the value is ignored; a NUL byte ends the text) and
// records where each top-level child starts and whether it is a number.
// One thread per (body, child) then converts the number exactly:
//   - w x 10^q with w < 2^53 and |q| <= 22: one correctly rounded IEEE
//     multiply or divide (both operands exact: Clinger's fast path);
//   - otherwise exact big-integer arithmetic: w x 10^q rounded to 53 bits
//     (q >= 0), or the quotient w x 2^s / 10^-q taken to 54+ bits with a
//     sticky remainder (q < 0), rounded half to even, with subnormals and
//     overflow to infinity as strtod gives them;
//   - more than 19 significant digits: w = the first 19 digits and w + 1
//     bound the value; if both round to the same double that is the result,
//     else the body is reported as not decodable (SVDB_DEC_UNSUPPORTED).
#include <cstring>
#include <mutex>
#include <new>

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
// characters; returns the characters consumed (0: no number).
__device__ int scan_number(const uint8_t* p, int n, Dec& d) {
    int run = 0;
    while (run < n && run < 63 && is_num_char(p[run])) ++run;
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

__device__ double to_double(const Dec& d, bool* ok) {
    *ok = true;
    if (d.zero || d.w == 0) return d.neg ? -0.0 : 0.0;
    if (!d.more) {
        if (d.w <= (1ull << 53) && d.q >= -22 && d.q <= 22) {
            double p = 1.0;
            for (int k = 0; k < (d.q < 0 ? -d.q : d.q); ++k) p *= 10.0;  // 10^k, k <= 22: exact
            const double x = (double)d.w;
            const double v = d.q >= 0 ? __dmul_rn(x, p) : __ddiv_rn(x, p);
            return d.neg ? -v : v;
        }
        return exact_value(d.w, d.q, d.neg);
    }
    // digits beyond the 19 kept: the value lies strictly between w and w + 1 units
    const double a = exact_value(d.w, d.q, d.neg);
    const double b = exact_value(d.w + 1, d.q, d.neg);
    if (__double_as_longlong(a) != __double_as_longlong(b)) *ok = false;
    return a;
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

__global__ void k_decode_parse(const uint8_t* __restrict__ text, const uint64_t* __restrict__ off, int nreq,
                               int64_t dim, int64_t* __restrict__ child, int32_t* __restrict__ status) {
    const int r = blockIdx.x * blockDim.x + threadIdx.x;
    if (r >= nreq) return;
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
                                 int64_t dim, const int64_t* __restrict__ child, int32_t* __restrict__ status,
                                 double* __restrict__ out) {
    const int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (t >= (int64_t)nreq * dim) return;
    const int64_t r = t / dim;
    if (status[r] != SVDB_DEC_OK) {
        out[t] = __longlong_as_double(0x7ff8000000000000ll);
        return;
    }
    const int64_t lo = (int64_t)off[r], hi = (int64_t)off[r + 1];
    const int64_t at = lo + child[t];
    Dec d;
    scan_number(text + at, hi - at < 64 ? (int)(hi - at) : 64, d);
    bool ok = true;
    out[t] = to_double(d, &ok);
    if (!ok) atomicExch(&status[r], SVDB_DEC_UNSUPPORTED);
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

}  // namespace

// Decode n bodies (host bytes text[off[i] .. off[i+1])) into n x dim doubles.
// Page-locked text and outputs are read and written by DMA directly; pageable
// ones go through the context's staging buffer.
int decode_bodies(Store* s, const char* text, const uint64_t* off, size_t n, size_t dim, double* out,
                  int32_t* status) {
    if (n == 0) return SVDB_OK;
    const size_t tb = off[n] - off[0];
    const size_t ob = (n + 1) * sizeof(uint64_t);
    const size_t cb = n * dim * sizeof(int64_t), vb = n * dim * sizeof(double), sb = n * sizeof(int32_t);
    const size_t a_text = round_up(tb + 1, 256), a_off = round_up(ob, 256), a_ch = round_up(cb, 256),
                 a_val = round_up(vb, 256);
    int rc = s->scratch_reserve(a_text + a_off + a_ch + a_val + sb + 256);
    if (!rc) rc = s->pinned_reserve(std::max(round_up(tb, 8) + ob, vb + sb));
    if (rc) return rc;
    uint8_t* base = (uint8_t*)s->scratch;
    uint8_t* dtext = base;
    uint64_t* doff = (uint64_t*)(base + a_text);
    int64_t* dch = (int64_t*)(base + a_text + a_off);
    double* dval = (double*)(base + a_text + a_off + a_ch);
    int32_t* dst = (int32_t*)(base + a_text + a_off + a_ch + a_val);
    uint8_t* hp = (uint8_t*)s->pin;
    const bool pin_in = host_pinned(text + off[0]);
    const bool pin_out = host_pinned(out) && host_pinned(status);
    if (!pin_in) std::memcpy(hp, text + off[0], tb);
    uint64_t* hoff = (uint64_t*)(hp + round_up(tb, 8));
    for (size_t i = 0; i <= n; ++i) hoff[i] = off[i] - off[0];
    SVDB_CUDA(cudaMemcpyAsync(dtext, pin_in ? (const void*)(text + off[0]) : (const void*)hp, tb,
                              cudaMemcpyHostToDevice, s->stream));
    SVDB_CUDA(cudaMemcpyAsync(doff, hoff, ob, cudaMemcpyHostToDevice, s->stream));
    k_decode_parse<<<(unsigned)((n + 63) / 64), 64, 0, s->stream>>>(dtext, doff, (int)n, (int64_t)dim, dch, dst);
    SVDB_LAUNCH_CHECK();
    const int64_t total = (int64_t)(n * dim);
    if (total)
        k_decode_numbers<<<(unsigned)((total + 255) / 256), 256, 0, s->stream>>>(dtext, doff, (int)n, (int64_t)dim, dch,
                                                                             dst, dval);
    SVDB_LAUNCH_CHECK();
    if (pin_out) {
        SVDB_CUDA(cudaMemcpyAsync(out, dval, vb, cudaMemcpyDeviceToHost, s->stream));
        SVDB_CUDA(cudaMemcpyAsync(status, dst, sb, cudaMemcpyDeviceToHost, s->stream));
        SVDB_CUDA(cudaStreamSynchronize(s->stream));
        return SVDB_OK;
    }
    SVDB_CUDA(cudaStreamSynchronize(s->stream));  // the pinned buffer is reused for the results
    SVDB_CUDA(cudaMemcpyAsync(hp, dval, vb, cudaMemcpyDeviceToHost, s->stream));
    SVDB_CUDA(cudaMemcpyAsync(hp + vb, dst, sb, cudaMemcpyDeviceToHost, s->stream));
    SVDB_CUDA(cudaStreamSynchronize(s->stream));
    std::memcpy(out, hp, vb);
    std::memcpy(status, hp + vb, sb);
    return SVDB_OK;
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
