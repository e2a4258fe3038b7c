// gen.h — the draws of the deterministic batch generators, shared by the host
// generator (gen.cpp) and the device generator (gen_dev.cu).
//
// One definition of every draw, so a batch made on the GPU is byte-identical
// to the host's.  Floating point (the Zipf sampler only) uses nothing but
// correctly rounded IEEE-754 double +, -, *, / and floor, with no contraction
// into fused multiply-adds (host: -ffp-contract=off; device: -fmad=false):
// those round the same on x86-64, aarch64 and the GPU.  Library pow / exp / log
// are not correctly rounded and differ between glibc and CUDA in the last ulp,
// so the sampler's power is computed below in fixed point, from tables filled
// by series of our own.
#pragma once
#include <string.h>

#include "proto.h"

#if defined(__CUDACC__)
#define LTPG_HDI __host__ __device__ inline
#else
#define LTPG_HDI inline
#endif

namespace ltpg {
namespace gen {

constexpr uint64_t DOM_YCSB_OPS = 0x59435342ull;   // "YCSB"
constexpr uint64_t DOM_YCSB_VAL = 0x56414C55ull;   // "VALU"
constexpr uint64_t DOM_YCSB_PERM = 0x5045524Dull;  // "PERM"
constexpr uint64_t DOM_TPCC = 0x54504343ull;       // "TPCC"

LTPG_HDI uint64_t mulhi64(uint64_t a, uint64_t b) {
#if defined(__CUDA_ARCH__)
    return __umul64hi(a, b);
#else
    return (uint64_t)(((unsigned __int128)a * b) >> 64);
#endif
}
LTPG_HDI uint64_t dbits(double x) {
#if defined(__CUDA_ARCH__)
    return (uint64_t)__double_as_longlong(x);
#else
    uint64_t b;
    memcpy(&b, &x, 8);
    return b;
#endif
}
LTPG_HDI double dfrom(uint64_t b) {
#if defined(__CUDA_ARCH__)
    return __longlong_as_double((long long)b);
#else
    double x;
    memcpy(&x, &b, 8);
    return x;
#endif
}
LTPG_HDI double dfloor(double x) {
#if defined(__CUDA_ARCH__)
    return floor(x);
#else
    return __builtin_floor(x);
#endif
}

// A transaction's splitmix64 stream.
struct Rng {
    uint64_t s;
    LTPG_HDI explicit Rng(uint64_t seed) : s(seed) {}
    LTPG_HDI uint64_t next() {
        s += 0x9E3779B97F4A7C15ull;
        uint64_t z = s;
        z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
        z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
        return z ^ (z >> 31);
    }
    // Uniform in [0, n) by Lemire's multiply-shift (integer only).
    LTPG_HDI uint64_t below(uint64_t n) { return mulhi64(next(), n); }
    // Uniform in [a, b].
    LTPG_HDI uint64_t range(uint64_t a, uint64_t b) { return a + below(b - a + 1); }
    LTPG_HDI double unit() { return (double)(next() >> 11) * 0x1.0p-53; }
};

// Bijection of [0, n) keyed by k: a 4-round Feistel network over the smallest
// even bit width covering n, with cycle walking back into range.
struct Perm {
    uint64_t n = 0, key = 0;
    uint32_t half = 1;
    LTPG_HDI void init(uint64_t n_, uint64_t key_) {
        n = n_;
        key = key_;
        uint32_t bits = 2;
        while (bits < 64 && (1ull << bits) < n) bits += 2;
        half = bits / 2;
    }
    LTPG_HDI uint64_t round_fn(uint64_t x, uint32_t r) const {
        return splitmix64(x ^ (key + 0x1234567ull * (r + 1))) & ((1ull << half) - 1);
    }
    LTPG_HDI uint64_t once(uint64_t x) const {
        const uint64_t m = (1ull << half) - 1;
        uint64_t l = x >> half, rr = x & m;
        for (uint32_t r = 0; r < 4; ++r) {
            uint64_t t = l ^ round_fn(rr, r);
            l = rr;
            rr = t;
        }
        return (l << half) | rr;
    }
    LTPG_HDI uint64_t operator()(uint64_t x) const {
        uint64_t y = once(x);
        while (y >= n) y = once(y);
        return y;
    }
};

// ---- power by series ------------------------------------------------------
// ln x for normal x > 0: x = m 2^e with m in [1/sqrt 2, sqrt 2), and
// ln m = 2 atanh(s) = 2 (s + s^3/3 + s^5/5 + ...), s = (m - 1) / (m + 1),
// |s| <= 0.1716 (the classical atanh series; eleven terms leave a relative
// error near 1e-16).  m - 1 is exact (Sterbenz).
constexpr double LN2 = 0.6931471805599453094;
constexpr double LN2_HI = 0.693147180369123816490;     // 32 significant bits: k * LN2_HI is exact
constexpr double LN2_LO = 1.90821492927058770002e-10;  // LN2 - LN2_HI
LTPG_HDI double det_log(double x) {
    const uint64_t b = dbits(x);
    int e = (int)((b >> 52) & 0x7FF) - 1023;
    double m = dfrom((b & 0x000FFFFFFFFFFFFFull) | 0x3FF0000000000000ull);  // [1, 2)
    if (m > 1.4142135623730951) {
        m = m * 0.5;
        e += 1;
    }
    const double s = (m - 1.0) / (m + 1.0);
    const double z = s * s;
    double p = 1.0 / 21.0;
    p = p * z + 1.0 / 19.0;
    p = p * z + 1.0 / 17.0;
    p = p * z + 1.0 / 15.0;
    p = p * z + 1.0 / 13.0;
    p = p * z + 1.0 / 11.0;
    p = p * z + 1.0 / 9.0;
    p = p * z + 1.0 / 7.0;
    p = p * z + 1.0 / 5.0;
    p = p * z + 1.0 / 3.0;
    p = p * z + 1.0;
    return (double)e * LN2 + 2.0 * s * p;
}
// e^y for y <= 0 (and small positive y): y = k ln 2 + r by Cody and Waite's
// two-constant reduction, |r| <= ln 2 / 2, e^r by its Taylor series to degree
// 14 (remainder below 1e-18), scaled by 2^k built from its exponent bits.
LTPG_HDI double det_exp(double y) {
    if (y < -745.0) return 0.0;
    const double k = dfloor(y * (1.0 / LN2) + 0.5);
    const double r = (y - k * LN2_HI) - k * LN2_LO;
    double p = 1.0 / 87178291200.0;   // 1/14!
    p = p * r + 1.0 / 6227020800.0;   // 1/13!
    p = p * r + 1.0 / 479001600.0;
    p = p * r + 1.0 / 39916800.0;
    p = p * r + 1.0 / 3628800.0;
    p = p * r + 1.0 / 362880.0;
    p = p * r + 1.0 / 40320.0;
    p = p * r + 1.0 / 5040.0;
    p = p * r + 1.0 / 720.0;
    p = p * r + 1.0 / 120.0;
    p = p * r + 1.0 / 24.0;
    p = p * r + 1.0 / 6.0;
    p = p * r + 0.5;
    p = p * r + 1.0;
    p = p * r + 1.0;
    int ki = (int)k;
    if (ki < -1022) {  // subnormal result: two exact-exponent steps
        p = p * dfrom((uint64_t)(1023 - 600) << 52);
        ki += 600;
    }
    return p * dfrom((uint64_t)(ki + 1023) << 52);
}
// x^a for x in (0, 1], a > 0; 0 for x <= 0 or x below the normal range.
LTPG_HDI double det_pow(double x, double a) {
    if (!(x >= 2.2250738585072014e-308)) return 0.0;
    return det_exp(a * det_log(x));
}

// ---- fixed-point power (the sampler's) -----------------------------------
// The sampler needs v = floor(n b^a) for b in (0, 1], a = 1 / (1 - theta) >= 1.
// It is computed in 64-bit fixed point (Q63: 1.0 = 2^63) by table-driven
// log2 and exp2 in the manner of Tang (ACM TOMS 1989/1990): b = m 2^-K,
// m = (1 + j/128)(1 + r), |r| < 2^-7, log2(1 + r) by the atanh-free series
// ln(1 + r) = r - r^2/2 + ... (nine terms); a log2(1/b) = I + k/64 + g,
// 2^-(k/64) from a table and 2^-g = e^(-g ln 2) by its Taylor series (eight
// terms).  Integer arithmetic only, so host and GPU give the same v by
// construction, and GB300's integer pipes run it about ten times faster than
// the double-precision evaluation (whose FP64 rate is low on this part).  The
// tables are filled once on the host from the series functions above.
struct FixTables {
    uint64_t log2c[128];  // log2(1 + j/128), Q63
    uint64_t rcp[128];    // floor((2^64 - 1) / (128 + j))
    uint64_t exp2n[64];   // 2^(-k/64), Q63
};
constexpr uint64_t Q63_ONE = 1ull << 63;
inline void fix_tables_fill(FixTables &t) {
    for (int j = 0; j < 128; ++j) {
        t.log2c[j] = (uint64_t)(det_log(1.0 + j / 128.0) / LN2 * 0x1p63);
        t.rcp[j] = ~0ull / (uint64_t)(128 + j);
    }
    for (int k = 0; k < 64; ++k) t.exp2n[k] = k == 0 ? Q63_ONE : (uint64_t)(det_exp(-k * (LN2 / 64.0)) * 0x1p63);
}
// (a b) >> 63 for Q63 operands whose product is below 2, the low bit dropped.
LTPG_HDI uint64_t q63mul(uint64_t a, uint64_t b) { return mulhi64(a, b) << 1; }
struct U128 {
    uint64_t hi, lo;
};
LTPG_HDI U128 mul64(uint64_t a, uint64_t b) { return U128{mulhi64(a, b), a * b}; }
LTPG_HDI uint64_t shr128(U128 x, uint32_t s) {  // (x >> s) mod 2^64, s < 128
    if (s == 0) return x.lo;
    if (s < 64) return (x.hi << (64 - s)) | (x.lo >> s);
    return x.hi >> (s - 64);
}
// floor(n b^a) for b in (0, 1] (normal), 1 <= a < 2^20, n < 2^40.
LTPG_HDI uint64_t fix_pow_floor(const FixTables &t, double b, double a, uint64_t n) {
    const uint64_t bb = dbits(b), ab = dbits(a);
    const uint32_t eb = (uint32_t)((bb >> 52) & 0x7FF), ea = (uint32_t)((ab >> 52) & 0x7FF);
    if (eb == 0 || eb > 1023) return eb > 1023 ? n : 0;  // b > 1 cannot occur; b subnormal -> 0
    const uint64_t M = (bb & 0x000FFFFFFFFFFFFFull) | (1ull << 52);
    const uint32_t j = (uint32_t)(M >> 45) - 128u;       // 0 .. 127
    const uint64_t D = M & ((1ull << 45) - 1);
    const uint64_t r = shr128(mul64(D, t.rcp[j]), 46);   // Q63, < 2^-7
    // ln(1 + r) = r (1 - r (1/2 - r (1/3 - ... - r/9))), every bracket positive
    uint64_t p = Q63_ONE / 9;
    p = Q63_ONE / 8 - q63mul(r, p);
    p = Q63_ONE / 7 - q63mul(r, p);
    p = Q63_ONE / 6 - q63mul(r, p);
    p = Q63_ONE / 5 - q63mul(r, p);
    p = Q63_ONE / 4 - q63mul(r, p);
    p = Q63_ONE / 3 - q63mul(r, p);
    p = Q63_ONE / 2 - q63mul(r, p);
    p = Q63_ONE - q63mul(r, p);
    const uint64_t inv_ln2 = (uint64_t)((1.0 / LN2) * 0x1p63);
    const uint64_t lm = t.log2c[j] + q63mul(q63mul(r, p), inv_ln2);  // log2 m, Q63, < 1
    // L = log2(1/b) = K - log2 m, K = 1023 - eb; as 128 bits in Q63
    const uint64_t K = 1023u - eb;
    const uint64_t lo0 = (K & 1u) << 63;
    U128 L{(K >> 1) - (lo0 < lm ? 1u : 0u), lo0 - lm};
    if (K == 0) L = U128{0, 0};  // b = 1 (then lm = 0)
    // Y = a L in Q63: a = Ma 2^(ea - 1075), Ma < 2^53
    const uint64_t Ma = (ab & 0x000FFFFFFFFFFFFFull) | (1ull << 52);
    const U128 pl = mul64(L.lo, Ma);
    const U128 prod{pl.hi + L.hi * Ma, pl.lo};
    const uint32_t s = 1075u - ea;  // 32 < s <= 52 for 1 <= a < 2^20
    const U128 Y{prod.hi >> s, (prod.hi << (64 - s)) | (prod.lo >> s)};
    if (Y.hi >= 64u) return 0;  // 2^-I with I >= 128
    const uint32_t I = (uint32_t)((Y.hi << 1) | (Y.lo >> 63));
    const uint64_t F = Y.lo & (Q63_ONE - 1);
    const uint32_t k = (uint32_t)(F >> 57);
    const uint64_t x = q63mul(F & ((1ull << 57) - 1), (uint64_t)(LN2 * 0x1p63));  // g ln 2 < 0.011
    // e^-x = 1 - x (1 - x (1/2 - x (1/6 - x (1/24 - x (1/120 - x (1/720 - x/5040))))))
    uint64_t e = Q63_ONE / 5040;
    e = Q63_ONE / 720 - q63mul(x, e);
    e = Q63_ONE / 120 - q63mul(x, e);
    e = Q63_ONE / 24 - q63mul(x, e);
    e = Q63_ONE / 6 - q63mul(x, e);
    e = Q63_ONE / 2 - q63mul(x, e);
    e = Q63_ONE - q63mul(x, e);
    e = Q63_ONE - q63mul(x, e);
    const uint64_t P = q63mul(t.exp2n[k], e);  // b^a 2^I, Q63, in (1/2, 1]
    const uint32_t sh = 63u + I;
    return sh >= 128u ? 0 : shr128(mul64(n, P), sh);
}

// Zipfian ranks by the method of Gray, Sundaresan, Englert, Baclawski and
// Weinberger, "Quickly generating billion-record synthetic databases" (SIGMOD
// 1994), the sampler YCSB uses.  Rank 0 is the most popular.  The constants
// are computed once on the host (zipf_init in gen.cpp).
struct Zipf {
    uint64_t n = 0;
    double theta = 0, zetan = 0, alpha = 0, eta = 0, half_pow = 0;
    LTPG_HDI uint64_t sample(Rng &r, const FixTables &tab) const {
        if (theta == 0.0) return r.below(n);
        const double u = r.unit();
        const double uz = u * zetan;
        if (uz < 1.0) return 0;
        if (uz < 1.0 + half_pow) return n > 1 ? 1 : 0;
        const uint64_t v = fix_pow_floor(tab, eta * u - eta + 1.0, alpha, n);
        return v < n ? v : n - 1;
    }
};

// Op words of YCSB transaction t of batch batch_id (distinct keys; a read
// scans scan_len keys when scan_len >= 2, its span in the field bits); pads to
// the op stride.  Returns the number of updates.
LTPG_HDI uint32_t ycsb_txn(const ltpg_ycsb_params &p, const Zipf &zipf, const FixTables &tab, const Perm *perm,
                           uint64_t batch_id, uint32_t t, uint32_t *w) {
    Rng r(hash3(p.seed ^ DOM_YCSB_OPS, batch_id, t));
    const uint32_t k = p.ops_per_txn, stride = ycsb_stride(k);
    uint32_t keys[LTPG_YCSB_MAX_OPS];
    uint32_t nupd = 0;
    for (uint32_t j = 0; j < k; ++j) {
        uint64_t key = 0;
        for (uint32_t attempt = 0;; ++attempt) {
            const uint64_t rank = zipf.sample(r, tab);
            key = perm ? (*perm)(rank) : rank;
            if (attempt >= 64) {  // pathological tiny tables: walk to a free key
                for (;;) {
                    bool dup = false;
                    for (uint32_t q = 0; q < j; ++q) dup |= keys[q] == key;
                    if (!dup) break;
                    key = (key + 1) % p.n_records;
                }
                break;
            }
            bool dup = false;
            for (uint32_t q = 0; q < j; ++q) dup |= keys[q] == key;
            if (!dup) break;
        }
        keys[j] = (uint32_t)key;
        const bool upd = r.below(100) < p.update_pct;
        const uint32_t field = (uint32_t)r.below(LTPG_YCSB_FIELDS);
        const uint32_t span = p.scan_len >= 2u ? p.scan_len - 1u : 0u;
        w[j] = ycsb_word((uint32_t)key, upd, upd ? field : span);
        nupd += upd;
    }
    for (uint32_t j = k; j < stride; ++j) w[j] = LTPG_YCSB_OP_PAD;
    return nupd;
}
LTPG_HDI uint64_t ycsb_value(const ltpg_ycsb_params &p, uint64_t txn, uint32_t j) {
    return hash3(p.seed ^ DOM_YCSB_VAL, txn, j);
}

// ---- TPC-C -----------------------------------------------------------------
// NURand of the reference, without the run-time constant C (Random.h:72-75).
LTPG_HDI uint64_t nurand(Rng &r, uint64_t A, uint64_t x, uint64_t y) {
    const uint64_t a = r.range(0, A);
    return ((a | r.range(x, y)) % (y - x + 1)) + x;
}
LTPG_HDI uint32_t other_w(Rng &r, uint32_t w, uint32_t W) {
    const uint32_t o = (uint32_t)r.below(W - 1);
    return o >= w ? o + 1 : o;
}

// The first draws of every transaction: kind (by the mix), home warehouse,
// district, and for a NewOrder its line count.
struct TpccHead {
    uint32_t kind, w, d, cnt;
};
LTPG_HDI TpccHead tpcc_head(const ltpg_tpcc_params &p, Rng &r) {
    TpccHead h;
    const uint32_t u = (uint32_t)r.below(100);
    h.w = (uint32_t)r.below(p.warehouses);
    h.d = (uint32_t)r.below(10);
    const uint32_t c_os = p.neworder_pct + p.orderstatus_pct, c_dl = c_os + p.delivery_pct,
                   c_sl = c_dl + p.stocklevel_pct;
    h.cnt = 0;
    if (u < p.neworder_pct) {
        h.kind = LTPG_TPCC_NEWORDER;
        h.cnt = (uint32_t)r.range(5, LTPG_TPCC_MAX_LINES);
    } else if (u < c_os) {
        h.kind = LTPG_TPCC_ORDERSTATUS;
    } else if (u < c_dl) {
        h.kind = LTPG_TPCC_DELIVERY;
    } else if (u < c_sl) {
        h.kind = LTPG_TPCC_STOCKLEVEL;
    } else {
        h.kind = LTPG_TPCC_PAYMENT;
    }
    return h;
}

// By last name (TF/Query.h:174-181): the query names customer (cw, cd, c_id)
// by its C_LAST and its rank among that name's holders in its district.
LTPG_HDI void tpcc_by_name(const ltpg_tpcc_params &p, Rng &r, ltpg_tpcc_txn &x, uint32_t cw, uint32_t cd,
                           const uint16_t *cust_name, const uint8_t *cust_rank) {
    if (p.by_name_pct && r.below(100) < p.by_name_pct) {
        const uint64_t row = 30000ull * cw + 3000ull * cd + x.c_id;
        if (cust_rank[row] < 255u) {
            x.kind_info |= LTPG_PAY_BY_NAME;
            x.c_id = ((uint32_t)cust_name[row] << 8) | cust_rank[row];
        }
    }
}

// NewOrder after its head: customer, then the lines (distinct items within an
// order, TF/Query.h:103-114).  O_ID / NO_ID / first OL_ID are the caller's.
LTPG_HDI void tpcc_neworder(const ltpg_tpcc_params &p, Rng &r, const TpccHead &h, ltpg_tpcc_txn &x,
                            ltpg_tpcc_line *lines) {
    x.kind_info = LTPG_TPCC_NEWORDER | (h.cnt << 8) | (h.d << 16);
    x.c_w = h.w;
    x.c_id = (uint32_t)nurand(r, 1023, 1, 3000) - 1;
    for (uint32_t i = 0; i < h.cnt; ++i) {
        uint32_t item;
        for (;;) {
            item = (uint32_t)nurand(r, 8191, 1, 100000) - 1;
            bool dup = false;
            for (uint32_t q = 0; q < i; ++q) dup |= lines[q].i_id == item;
            if (!dup) break;
        }
        ltpg_tpcc_line ln;
        ln.i_id = item;
        const bool remote = p.warehouses > 1 && r.below(100) < p.remote_line_pct;
        ln.supply_w = (uint16_t)(remote ? other_w(r, h.w, p.warehouses) : h.w);
        ln.qty = (uint16_t)r.range(1, 10);
        lines[i] = ln;
    }
}

// Payment after its head; H_ID is the caller's.
LTPG_HDI void tpcc_payment(const ltpg_tpcc_params &p, Rng &r, const TpccHead &h, ltpg_tpcc_txn &x,
                           const uint16_t *cust_name, const uint8_t *cust_rank) {
    const bool remote = p.warehouses > 1 && r.below(100) < p.remote_pay_pct;
    uint32_t c_w = h.w, c_d = h.d;
    if (remote) {
        c_w = other_w(r, h.w, p.warehouses);
        c_d = (uint32_t)r.below(10);
    }
    x.kind_info = LTPG_TPCC_PAYMENT | (h.d << 16) | (c_d << 24);
    x.c_w = c_w;
    x.c_id = (uint32_t)nurand(r, 1023, 1, 3000) - 1;
    const uint64_t amount = r.range(100, 500000);
    x.b = (uint32_t)amount;
    x.c = (uint32_t)(amount >> 32);
    tpcc_by_name(p, r, x, c_w, c_d, cust_name, cust_rank);
}

// StockLevel after its head (TA/Query.h:270-296): one stock row of w.
LTPG_HDI void tpcc_stocklevel(Rng &r, const TpccHead &h, ltpg_tpcc_txn &x) {
    const uint32_t threshold = (uint32_t)r.range(10, 20);
    x.kind_info = LTPG_TPCC_STOCKLEVEL | (threshold << 8) | (h.d << 16);
    x.c_w = h.w;
    x.a = (uint32_t)nurand(r, 8191, 1, 100000) - 1;
}

// A tracked order as the generator remembers it.
struct TpccOrder {
    uint32_t cust, dist, ol, cnt;
};

// OrderStatus after its head (TA/Query.h:214-246): a recent order of warehouse
// w and one of its lines, read with its customer.  made = orders warehouse w
// has made so far (0 when untracked), o_id = its next O_ID; order(o) returns
// the tracked order with O_ID o.
template <class Lookup>
LTPG_HDI void tpcc_orderstatus(const ltpg_tpcc_params &p, Rng &r, const TpccHead &h, ltpg_tpcc_txn &x, uint64_t made,
                               uint32_t o_id, Lookup order, const uint16_t *cust_name, const uint8_t *cust_rank) {
    uint32_t cd = h.d, o, ol;
    if (made) {
        const uint64_t back = r.below(made < 1000 ? made : 1000);
        o = (uint32_t)((o_id + 30000u - 1u - (uint32_t)back) % 30000u);
        const TpccOrder od = order(o);
        cd = od.dist;
        x.c_id = od.cust;
        ol = (uint32_t)((od.ol + r.below(od.cnt > 1u ? od.cnt : 1u)) % 450000u);
    } else {
        x.c_id = (uint32_t)nurand(r, 1023, 1, 3000) - 1;
        o = (uint32_t)r.below(30000);
        ol = (uint32_t)r.below(450000);
    }
    x.kind_info = LTPG_TPCC_ORDERSTATUS | (cd << 16) | (cd << 24);
    x.c_w = h.w;
    x.a = o;
    x.b = ol;
    tpcc_by_name(p, r, x, h.w, cd, cust_name, cust_rank);
}

// Delivery after its head (TA/Query.h:247-269): the oldest undelivered order
// of w when `tracked` (its O_ID o, chosen by the caller), else a random one.
template <class Lookup>
LTPG_HDI void tpcc_delivery(Rng &r, const TpccHead &h, ltpg_tpcc_txn &x, bool tracked, uint32_t o, Lookup order) {
    uint32_t cd = h.d, ol;
    if (tracked) {
        const TpccOrder od = order(o);
        cd = od.dist;
        x.c_id = od.cust;
        ol = od.ol;
    } else {
        x.c_id = (uint32_t)nurand(r, 1023, 1, 3000) - 1;
        o = (uint32_t)r.below(30000);
        ol = (uint32_t)r.below(450000);
    }
    const uint32_t carrier = (uint32_t)r.range(1, 10);
    x.kind_info = LTPG_TPCC_DELIVERY | (carrier << 8) | (cd << 16);
    x.c_w = h.w;
    x.a = o;
    x.b = o;  // NO_ID and O_ID advance together (TF/Query.h:54-88)
    x.c = ol;
}

}  // namespace gen
}  // namespace ltpg
