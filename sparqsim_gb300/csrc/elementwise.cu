// elementwise.cu — the fused elementwise kernel.
//
// Every reference operator whose CPU loop touches one entry at a time
// (register arithmetic, QRAM gather, phases, in-place rotations) is one
// instruction of a small program. One launch streams the state once: each
// thread loads the key words the program reads (and the amplitude if any
// instruction needs it), runs the instructions in order with their own
// control conditions, and stores only what changed. Consecutive operators
// therefore cost one HBM pass instead of one pass each, and the reference's
// partition-by-condition pass (cuda/system_operations.cu:17-66) disappears
// because conditions are evaluated per entry in registers.
#include <algorithm>
#include <cstring>

#include "sq_internal.cuh"

namespace sq {

// A register field with its masks computed on the host, so that a field
// access costs a word select, a shift and an AND per entry
struct DField {
    uint8_t word;
    uint8_t shift;
    uint8_t width;
    uint8_t type;
    uint32_t pad;
    uint64_t mask;   // wmask(width)
    uint64_t smask;  // mask << shift
};
static DField dfield(const Field& f) {
    DField d;
    d.word = f.word;
    d.shift = f.shift;
    d.width = f.width;
    d.type = f.type;
    d.pad = 0;
    d.mask = wmask(f.width);
    d.smask = d.mask << f.shift;
    return d;
}
template <int K>
__device__ __forceinline__ uint64_t fget(const uint64_t (&k)[K], const DField& f) {
    return (kword<K>(k, f.word) >> f.shift) & f.mask;
}
template <int K>
__device__ __forceinline__ void fset(uint64_t (&k)[K], const DField& f, uint64_t v) {
    const uint64_t w = kword<K>(k, f.word);
    kword_set<K>(k, f.word, (w & ~f.smask) | ((v << f.shift) & f.smask));
}

struct DInstr {
    uint16_t op;
    uint8_t dag;
    uint8_t pad;
    uint32_t addr_bits;
    uint64_t amask;  // wmask(addr_bits)
    DField f[4];
    uint64_t imm[3];
    double2 c[2];
    const void* table;
    uint32_t elem_bytes;
    uint32_t pad2;
    uint64_t zmask[SQ_KMAX];
    DCondSet cond;
};

template <int MAXI>
struct ProgramArgs {
    unsigned* err;         // device error word (bit 3: a lookup value without a table entry)
    uint32_t n;
    uint32_t read_words;   // bit w: word w is read
    uint32_t write_words;  // bit w: word w is written
    uint32_t amp_mode;     // bit 0: read amplitude, bit 1: write amplitude
    DInstr ins[MAXI];
};

__device__ __forceinline__ int64_t sext(uint64_t v, unsigned w) {
    if (w == 0) return 0;
    if (w >= 64) return (int64_t)v;
    const uint64_t sign = 1ull << (w - 1);
    return (int64_t)((v ^ sign) - sign);
}

__device__ __forceinline__ uint64_t isqrt64(uint64_t v) {
    uint64_t res = 0, bit = 1ull << 62;
    while (bit > v) bit >>= 2;
    while (bit) {
        if (v >= res + bit) {
            v -= res + bit;
            res = (res >> 1) + bit;
        } else {
            res >>= 1;
        }
        bit >>= 2;
    }
    return res;
}

// complex multiply without contraction (the library is built with --fmad=false)
__device__ __forceinline__ double2 cmul(double2 a, double2 b) {
    return make_double2(a.x * b.x - a.y * b.y, a.x * b.y + a.y * b.x);
}

__device__ __forceinline__ uint64_t shl(uint64_t v, unsigned s) { return s >= 64 ? 0 : v << s; }
__device__ __forceinline__ uint64_t shr(uint64_t v, unsigned s) { return s >= 64 ? 0 : v >> s; }

// The combined [elements | column indices] table of a constant-diagonal
// tridiagonal matrix with 4-slot row windows, computed instead of stored
// (hamiltonian_simulation_tridiagonal.h:104-190): row j's window starts at
// clamp(j - 1, 0, n - 4); enc = alpha_enc | beta_enc << 32.
__device__ __forceinline__ uint64_t tri_window_base(uint64_t j, uint64_t n) {
    const uint64_t b = j > 0 ? j - 1 : 0, bmax = n - 4;
    return b < bmax ? b : bmax;
}
__device__ __forceinline__ uint64_t tri_mem(uint64_t idx, uint64_t n, uint64_t enc) {
    idx &= 8 * n - 1;
    const uint64_t half = 4 * n;
    if (idx < half) {
        const uint64_t j = idx >> 2, c = tri_window_base(j, n) + (idx & 3);
        if (c == j) return enc & 0xffffffffull;
        if (c + 1 == j || c == j + 1) return enc >> 32;
        return 0;
    }
    const uint64_t t = idx - half;
    return tri_window_base(t >> 2, n) + (t & 3);
}

// Parallel bit extract / deposit over the set bits of m, lowest first.
__device__ __forceinline__ uint64_t bits_extract(uint64_t v, uint64_t m) {
    uint64_t out = 0, b = 1;
    for (; m; m &= m - 1, b <<= 1)
        if (v & (m & (0ull - m))) out |= b;
    return out;
}
__device__ __forceinline__ uint64_t bits_deposit(uint64_t v, uint64_t m) {
    uint64_t out = 0, b = 1;
    for (; m; m &= m - 1, b <<= 1)
        if (v & b) out |= m & (0ull - m);
    return out;
}

template <int K>
__device__ __forceinline__ void exec(const DInstr& in, uint64_t (&k)[K], double2& a, unsigned* err) {
    const DField* f = in.f;
    switch (in.op) {
        case SQ_OP_FLIP_BOOLS: fset<K>(k, f[0], ~fget<K>(k, f[0])); break;
        case SQ_OP_SWAP_BOOL_BOOL: {
            uint64_t x = fget<K>(k, f[0]), y = fget<K>(k, f[1]);
            const uint64_t d1 = in.imm[0], d2 = in.imm[1];
            const bool v1 = (x >> d1) & 1, v2 = (y >> d2) & 1;
            if (v1 && !v2) { x -= 1ull << d1; y += 1ull << d2; }
            if (v2 && !v1) { x += 1ull << d1; y -= 1ull << d2; }
            fset<K>(k, f[0], x);
            fset<K>(k, f[1], y);
            break;
        }
        case SQ_OP_SHIFT_LEFT:
        case SQ_OP_SHIFT_RIGHT: {
            const unsigned size = f[0].width;
            const unsigned d = (unsigned)in.imm[0];
            const bool left = (in.op == SQ_OP_SHIFT_LEFT) != (in.dag != 0);
            const uint64_t v = fget<K>(k, f[0]);
            uint64_t r;
            if (left) {
                const uint64_t high = shr(v, size - d);
                const uint64_t low = v - shl(high, size - d);
                r = shl(low, d) + high;
            } else {
                const uint64_t high = shr(v, d);
                const uint64_t low = v - shl(high, d);
                r = shl(low, size - d) + high;
            }
            fset<K>(k, f[0], r);
            break;
        }
        case SQ_OP_MULT_UINT_CONST: fset<K>(k, f[2], fget<K>(k, f[2]) ^ (fget<K>(k, f[0]) * in.imm[0])); break;
        case SQ_OP_ADD_MULT_UINT_CONST: {
            const uint64_t o = fget<K>(k, f[2]), l = fget<K>(k, f[0]);
            fset<K>(k, f[2], in.dag ? o - l * in.imm[0] : o + in.imm[0] * l);
            break;
        }
        case SQ_OP_MOD_MULT_CONST: fset<K>(k, f[0], (fget<K>(k, f[0]) * in.imm[0]) % in.imm[1]); break;
        case SQ_OP_ADD_UINT_UINT: fset<K>(k, f[2], fget<K>(k, f[2]) ^ (fget<K>(k, f[0]) + fget<K>(k, f[1]))); break;
        case SQ_OP_ADD_UINT_UINT_INPLACE: {
            const uint64_t o = fget<K>(k, f[1]), l = fget<K>(k, f[0]);
            fset<K>(k, f[1], in.dag ? o - l : o + l);
            break;
        }
        case SQ_OP_ADD_UINT_CONST: fset<K>(k, f[2], fget<K>(k, f[2]) ^ (fget<K>(k, f[0]) + in.imm[0])); break;
        case SQ_OP_ADD_CONST_INPLACE: {
            const uint64_t o = fget<K>(k, f[0]);
            fset<K>(k, f[0], in.dag ? o - in.imm[0] : o + in.imm[0]);
            break;
        }
        case SQ_OP_PLUS_ONE_OVERFLOW: {
            const uint64_t v = fget<K>(k, f[0]);
            const uint64_t top = wmask(f[0].width);
            const bool wrap = in.dag ? v == 0 : v == top;
            fset<K>(k, f[0], in.dag ? v - 1 : v + 1);  // stored modulo 2^width
            if (wrap) fset<K>(k, f[1], (fget<K>(k, f[1]) + 1) % 2);
            break;
        }
        case SQ_OP_BIT_GATHER: {
            const uint64_t v = fget<K>(k, f[0]);
            const uint64_t set = in.imm[0], rest = wmask(f[0].width) & ~set;  // host: set below the width
            const unsigned ns = (unsigned)__popcll(set);
            fset<K>(k, f[0], in.dag ? bits_deposit(v, set) | bits_deposit(shr(v, ns), rest)
                                    : bits_extract(v, set) | shl(bits_extract(v, rest), ns));
            break;
        }
        case SQ_OP_SUB_UINT_UINT: fset<K>(k, f[2], fget<K>(k, f[2]) ^ (fget<K>(k, f[0]) - fget<K>(k, f[1]))); break;
        case SQ_OP_NEG_UINT: fset<K>(k, f[1], fget<K>(k, f[1]) ^ (0ull - fget<K>(k, f[0]))); break;
        case SQ_OP_ABS_SINT: {
            const int64_t v = sext(fget<K>(k, f[0]), f[0].width);
            const uint64_t mag = v < 0 ? (uint64_t)(-v) : (uint64_t)v;
            fset<K>(k, f[1], fget<K>(k, f[1]) ^ mag);
            break;
        }
        case SQ_OP_MUL_UINT_UINT: fset<K>(k, f[2], fget<K>(k, f[2]) ^ (fget<K>(k, f[0]) * fget<K>(k, f[1]))); break;
        case SQ_OP_DIV_UINT_UINT: {
            const uint64_t x = fget<K>(k, f[0]), y = fget<K>(k, f[1]);
            fset<K>(k, f[2], fget<K>(k, f[2]) ^ (y == 0 ? 0ull : x / y));
            break;
        }
        case SQ_OP_SQRT_UINT: fset<K>(k, f[1], fget<K>(k, f[1]) ^ isqrt64(fget<K>(k, f[0]))); break;
        case SQ_OP_SELECT_BOOL: {
            const uint64_t sel = (fget<K>(k, f[0]) & 1ull) ? fget<K>(k, f[1]) : fget<K>(k, f[2]);
            fset<K>(k, f[3], fget<K>(k, f[3]) ^ sel);
            break;
        }
        case SQ_OP_AND_UINT_UINT: fset<K>(k, f[2], fget<K>(k, f[2]) ^ (fget<K>(k, f[0]) & fget<K>(k, f[1]))); break;
        case SQ_OP_OR_UINT_UINT: fset<K>(k, f[2], fget<K>(k, f[2]) ^ (fget<K>(k, f[0]) | fget<K>(k, f[1]))); break;
        case SQ_OP_XOR_UINT_UINT: fset<K>(k, f[2], fget<K>(k, f[2]) ^ (fget<K>(k, f[0]) ^ fget<K>(k, f[1]))); break;
        case SQ_OP_LESS_SINT_SINT: {
            const bool p = sext(fget<K>(k, f[0]), f[0].width) < sext(fget<K>(k, f[1]), f[1].width);
            fset<K>(k, f[2], fget<K>(k, f[2]) ^ (p ? 1ull : 0ull));
            break;
        }
        case SQ_OP_CARRY_UINT_UINT: {
            const uint64_t x = fget<K>(k, f[0]), y = fget<K>(k, f[1]);
            const unsigned w = f[2].width;
            const bool p = w >= 64 ? (x + y < x) : (x >= (1ull << w)) || (y >= (1ull << w) - x);
            fset<K>(k, f[3], fget<K>(k, f[3]) ^ (p ? 1ull : 0ull));
            break;
        }
        case SQ_OP_OVERFLOW_SINT_SINT: {
            const unsigned w = f[2].width;
            const uint64_t m = wmask(w);
            const uint64_t A = (uint64_t)sext(fget<K>(k, f[0]), f[0].width) & m;
            const uint64_t B = (uint64_t)sext(fget<K>(k, f[1]), f[1].width) & m;
            const uint64_t S = (A + B) & m;
            const uint64_t sa = (A >> (w - 1)) & 1, sb = (B >> (w - 1)) & 1, ss = (S >> (w - 1)) & 1;
            const bool p = (sa == sb) && (ss != sa);
            fset<K>(k, f[3], fget<K>(k, f[3]) ^ (p ? 1ull : 0ull));
            break;
        }
        case SQ_OP_MULOVERFLOW_UINT_UINT: {
            const uint64_t x = fget<K>(k, f[0]), y = fget<K>(k, f[1]);
            const uint64_t lo = x * y, hi = __umul64hi(x, y);
            const unsigned w = f[2].width;
            const bool p = hi != 0 || (w < 64 && lo >= (1ull << w));
            fset<K>(k, f[3], fget<K>(k, f[3]) ^ (p ? 1ull : 0ull));
            break;
        }
        case SQ_OP_ISZERO_UINT: fset<K>(k, f[1], fget<K>(k, f[1]) ^ (fget<K>(k, f[0]) == 0 ? 1ull : 0ull)); break;
        case SQ_OP_NEGATIVE_SINT:
            fset<K>(k, f[1], fget<K>(k, f[1]) ^ (sext(fget<K>(k, f[0]), f[0].width) < 0 ? 1ull : 0ull));
            break;
        case SQ_OP_ADD_ANYINT_INPLACE: {
            const uint64_t raw = fget<K>(k, f[1]);
            const uint64_t ext = f[1].type == SQ_SIGNED ? (uint64_t)sext(raw, f[1].width) : raw;
            const uint64_t o = fget<K>(k, f[0]);
            fset<K>(k, f[0], in.dag ? o - ext : o + ext);
            break;
        }
        case SQ_OP_ASSIGN: fset<K>(k, f[1], fget<K>(k, f[1]) ^ fget<K>(k, f[0])); break;
        case SQ_OP_COMPARE_UINT_UINT: {
            const uint64_t l = fget<K>(k, f[0]), r = fget<K>(k, f[1]);
            if (l == r) fset<K>(k, f[3], fget<K>(k, f[3]) ^ 1ull);
            else fset<K>(k, f[2], fget<K>(k, f[2]) ^ (l < r ? 1ull : 0ull));
            break;
        }
        case SQ_OP_LESS_UINT_UINT:
            fset<K>(k, f[2], fget<K>(k, f[2]) ^ (fget<K>(k, f[0]) < fget<K>(k, f[1]) ? 1ull : 0ull));
            break;
        case SQ_OP_SWAP_GENERAL: {
            const uint64_t x = fget<K>(k, f[0]), y = fget<K>(k, f[1]);
            fset<K>(k, f[0], y);
            fset<K>(k, f[1], x);
            break;
        }
        case SQ_OP_GETMID_UINT_UINT:
            fset<K>(k, f[2], fget<K>(k, f[2]) ^ ((fget<K>(k, f[0]) + fget<K>(k, f[1])) / 2));
            break;
        case SQ_OP_X_BOOL: fset<K>(k, f[0], fget<K>(k, f[0]) ^ (1ull << in.imm[0])); break;
        case SQ_OP_INIT_UNSAFE: fset<K>(k, f[0], in.imm[0]); break;
        case SQ_OP_QRAM_LOAD: {
            const uint64_t addr = fget<K>(k, f[0]) & in.amask;
            uint64_t word;
            if (in.elem_bytes == 2) word = __ldg((const unsigned short*)in.table + addr);
            else if (in.elem_bytes == 4) word = __ldg((const unsigned int*)in.table + addr);
            else word = __ldg((const unsigned long long*)in.table + addr);
            fset<K>(k, f[1], fget<K>(k, f[1]) ^ word);
            break;
        }
        case SQ_OP_ADDR_XOR: {
            uint64_t v = fget<K>(k, f[0]) + in.imm[0] * fget<K>(k, f[1]);
            if (in.imm[1]) v += fget<K>(k, f[2]);
            fset<K>(k, f[3], fget<K>(k, f[3]) ^ v);
            break;
        }
        case SQ_OP_QBS_XOR: {
            const uint64_t amask = wmask(in.addr_bits);
            const uint64_t target = fget<K>(k, f[1]);
            uint64_t l = fget<K>(k, f[0]), r = l + in.imm[0], found = 0;
            for (uint64_t i = 0; i < in.imm[1]; ++i) {
                const uint64_t mid = (l + r) / 2;
                uint64_t word;
                if (in.elem_bytes == 2) word = __ldg((const unsigned short*)in.table + (mid & amask));
                else if (in.elem_bytes == 4) word = __ldg((const unsigned int*)in.table + (mid & amask));
                else word = __ldg((const unsigned long long*)in.table + (mid & amask));
                if (word == target) {
                    found = mid;
                    break;
                }
                if (word < target) l = mid;
                else r = mid;
            }
            fset<K>(k, f[2], fget<K>(k, f[2]) ^ found);
            break;
        }
        case SQ_OP_TRIDIAG_ELEMENT: {
            const uint64_t idx = fget<K>(k, f[0]) + 4 * fget<K>(k, f[1]) + fget<K>(k, f[2]);
            fset<K>(k, f[3], fget<K>(k, f[3]) ^ tri_mem(idx, in.imm[0], in.imm[1]));
            break;
        }
        case SQ_OP_TRIDIAG_SLOT_COLUMN: {
            const uint64_t n = in.imm[0], kmask = wmask((unsigned)in.imm[2]);
            const uint64_t j = fget<K>(k, f[1]), kv = fget<K>(k, f[2]), sr = fget<K>(k, f[3]) & kmask;
            const uint64_t base = tri_window_base(j, n), row = fget<K>(k, f[0]) + 4 * j;
            if (!in.dag) {  // column -> slot; out-of-window branches tagged into the tag register
                const bool hit = kv >= base && kv < base + 4;
                const uint64_t sr1 = sr ^ (hit ? row + (kv - base) : 0ull);
                const uint64_t k1 = kv ^ tri_mem(sr1, n, in.imm[1]);
                fset<K>(k, f[2], (sr1 - row) & kmask);
                fset<K>(k, f[3], k1 & kmask);
            } else {  // slot -> column
                const uint64_t k1 = (kv + row) & kmask;
                const uint64_t k2 = sr ^ tri_mem(k1, n, in.imm[1]);
                const bool hit = k2 >= base && k2 < base + 4;
                fset<K>(k, f[2], k2);
                fset<K>(k, f[3], k1 ^ (hit ? row + (k2 - base) : 0ull));
            }
            break;
        }
        case SQ_OP_LOOKUP_XOR: {
            const uint64_t v = fget<K>(k, f[0]);
            const uint64_t* t = static_cast<const uint64_t*>(in.table);
            const uint64_t nd = in.imm[0], ns = in.imm[1];
            uint64_t w = 0;
            if (v < nd) {
                w = __ldg(t + v);
            } else {
                uint64_t lo = 0, hi = ns;
                while (lo < hi) {
                    const uint64_t mid = (lo + hi) >> 1;
                    if (__ldg(t + nd + mid) < v) lo = mid + 1;
                    else hi = mid;
                }
                if (lo < ns && __ldg(t + nd + lo) == v) w = __ldg(t + nd + ns + lo);
                else atomicOr(err, 8u);
            }
            fset<K>(k, f[1], fget<K>(k, f[1]) ^ w);
            break;
        }
        case SQ_OP_PARITY_PHASE:
            if (fget<K>(k, f[0]) & 1ull) a = make_double2(-a.x, -a.y);
            break;
        case SQ_OP_ANGLE_XOR: {
            const uint64_t l = fget<K>(k, f[0]), r = fget<K>(k, f[1]);
            const uint64_t* t = static_cast<const uint64_t*>(in.table);
            const uint64_t mask = in.imm[0];
            const unsigned probes = (unsigned)in.imm[1];
            const uint64_t h = pair_slot_hash(l, r);
            uint64_t w = 0;
            bool found = false;
            for (unsigned i = 0; i <= probes; ++i) {
                const uint64_t* slot = t + 3 * ((h + i) & mask);
                const uint64_t x = __ldg(slot), y = __ldg(slot + 1);
                if (x == l && y == r) {
                    w = __ldg(slot + 2);
                    found = true;
                    break;
                }
                if (x == ~0ull && y == ~0ull) break;
            }
            if (!found) atomicOr(err, 64u);
            fset<K>(k, f[2], fget<K>(k, f[2]) ^ w);
            break;
        }
        case SQ_OP_PHASE_BOOL:
            if ((fget<K>(k, f[0]) >> in.imm[0]) & 1ull) a = cmul(a, in.c[0]);
            break;
        case SQ_OP_GLOBAL_PHASE: a = cmul(a, in.c[0]); break;
        case SQ_OP_Y_BOOL: {
            const uint64_t v = fget<K>(k, f[0]) ^ (1ull << in.imm[0]);
            fset<K>(k, f[0], v);
            a = cmul(a, ((v >> in.imm[0]) & 1ull) ? make_double2(0.0, 1.0) : make_double2(0.0, -1.0));
            break;
        }
        case SQ_OP_REFLECTION_BOOL:
        case SQ_OP_ZERO_COND_PHASE_FLIP: {
            bool iszero = true;
#pragma unroll
            for (int w = 0; w < K; ++w) iszero = iszero && ((k[w] & in.zmask[w]) == 0);
            bool flip = in.op == SQ_OP_ZERO_COND_PHASE_FLIP ? iszero : !((in.imm[1] != 0) ^ iszero);
            if (flip) a = make_double2(a.x * -1.0, a.y * -1.0);
            break;
        }
        case SQ_OP_ROT_DIAGONAL:
            a = cmul(a, ((fget<K>(k, f[0]) >> in.imm[0]) & 1ull) ? in.c[1] : in.c[0]);
            break;
        case SQ_OP_ROT_OFF_DIAGONAL: {
            const uint64_t v = fget<K>(k, f[0]);
            a = cmul(a, ((v >> in.imm[0]) & 1ull) ? in.c[1] : in.c[0]);
            fset<K>(k, f[0], v ^ (1ull << in.imm[0]));
            break;
        }
        case SQ_OP_PAULI_NOISE: {
            const uint64_t t = fget<K>(k, f[0]);
            if (t >= in.imm[0]) break;
            uint64_t m[6];
#pragma unroll
            for (int r = 0; r < 6; ++r) {
                const uint64_t idx = t * 6 + r;
                if (in.elem_bytes == 2) m[r] = __ldg((const unsigned short*)in.table + idx);
                else if (in.elem_bytes == 4) m[r] = __ldg((const unsigned int*)in.table + idx);
                else m[r] = __ldg((const unsigned long long*)in.table + idx);
            }
            int parity = 0;
#pragma unroll
            for (int r = 0; r < 3; ++r) {
                const uint64_t v = fget<K>(k, f[r + 1]) ^ m[r];
                fset<K>(k, f[r + 1], v);
                parity += __popcll(v & m[r + 3]);
            }
            if (parity & 1) a = make_double2(a.x * -1.0, a.y * -1.0);
            break;
        }
        default: break;
    }
}

template <int K, int MAXI>
__global__ void __launch_bounds__(256) program_kernel(const __grid_constant__ ProgramArgs<MAXI> p, KeyPtrs keys,
                                                      double2* __restrict__ amp, uint64_t n) {
    // warp-uniform trips (the entry index is per lane, the loop is not), so
    // that the instruction index is uniform and the instruction's fields are
    // uniform loads
    const uint64_t stride = (uint64_t)gridDim.x * blockDim.x;
    for (uint64_t b = (uint64_t)blockIdx.x * blockDim.x; b < n; b += stride) {
        const uint64_t i = b + threadIdx.x;
        const bool valid = i < n;
        uint64_t k[K];
#pragma unroll
        for (int w = 0; w < K; ++w) k[w] = (valid && ((p.read_words >> w) & 1u)) ? keys.w[w][i] : 0ull;
        double2 a = make_double2(0.0, 0.0);
        if (valid && (p.amp_mode & 1u)) a = amp[i];
        for (uint32_t j = 0; j < p.n; ++j) {
            const DInstr& in = p.ins[j];
            if (valid && cond_ok<K>(k, in.cond)) exec<K>(in, k, a, p.err);
        }
        if (!valid) continue;
#pragma unroll
        for (int w = 0; w < K; ++w)
            if ((p.write_words >> w) & 1u) keys.w[w][i] = k[w];
        if (p.amp_mode & 2u) amp[i] = a;
    }
}

template <int K, int MAXI>
static void launch_program(const ProgramArgs<MAXI>& args, State& s, double table_bytes) {
    KeyPtrs kp;
    for (int w = 0; w < SQ_KMAX; ++w) kp.w[w] = s.live.keys[w];
    const int block = 256;
    unsigned grid = grid_for(s.n, block, 8);
    prof_begin("elementwise_program");
    program_kernel<K, MAXI><<<grid, block, 0, stream()>>>(args, kp, s.live.amp, s.n);
    // compulsory traffic: words read + words written + amplitude in/out + table words touched
    const double per = 8.0 * __builtin_popcount(args.read_words) + 8.0 * __builtin_popcount(args.write_words) +
                       16.0 * (args.amp_mode & 1u) + 16.0 * ((args.amp_mode >> 1) & 1u);
    prof_end((double)s.n * per + table_bytes);
    SQ_CUDA(cudaGetLastError());
}

template <int MAXI>
static void dispatch_k(const ProgramArgs<MAXI>& args, State& s, uint32_t k) {
    double tb = 0.0;
    for (uint32_t i = 0; i < args.n; ++i)
        if (args.ins[i].op == SQ_OP_QRAM_LOAD) {
            const double words = (double)(1ull << args.ins[i].addr_bits);
            tb += std::min((double)s.n, words) * args.ins[i].elem_bytes;
        }
    switch (k) {
        case 1: launch_program<1, MAXI>(args, s, tb); break;
        case 2: launch_program<2, MAXI>(args, s, tb); break;
        case 3: launch_program<3, MAXI>(args, s, tb); break;
        case 4: launch_program<4, MAXI>(args, s, tb); break;
        case 5: launch_program<5, MAXI>(args, s, tb); break;
        case 6: launch_program<6, MAXI>(args, s, tb); break;
        case 7: launch_program<7, MAXI>(args, s, tb); break;
        default: launch_program<8, MAXI>(args, s, tb); break;
    }
}

// ------------------------------------------------------------------ host-side translation
static uint32_t word_bit(const Field& f) { return f.width ? (1u << f.word) : 0u; }

static void need_regs(const sq_instr& in, int n) {
    for (int i = 0; i < n; ++i) (void)regtable().at(in.reg[i]);
}

static void distinct(uint32_t a, uint32_t b, const char* what) {
    if (a == b) fail(SQ_ERR_INVALID, std::string(what) + ": registers must be distinct");
}

// Translate one ABI instruction; returns (read words, write words, amp mode).
static void translate(const sq_instr& in, DInstr& d, uint32_t& rw, uint32_t& ww, uint32_t& am) {
    memset(&d, 0, sizeof(d));
    d.op = (uint16_t)in.op;
    d.dag = in.dag ? 1 : 0;
    d.imm[0] = in.imm[0];
    d.imm[1] = in.imm[1];
    d.imm[2] = in.imm[2];
    d.c[0] = make_double2(in.c[0], in.c[1]);
    d.c[1] = make_double2(in.c[2], in.c[3]);
    d.cond = resolve_cond(&in.cond);
    for (uint32_t i = 0; i < d.cond.n; ++i) rw |= 1u << d.cond.c[i].word;
    RegTable& t = regtable();
    auto F = [&](int slot) {
        const Field f = t.field(in.reg[slot]);
        d.f[slot] = dfield(f);
        return f;
    };
    auto R = [&](int slot) { rw |= word_bit(F(slot)); };
    auto W = [&](int slot) {
        Field f = F(slot);
        rw |= word_bit(f);
        ww |= word_bit(f);
    };
    switch (in.op) {
        case SQ_OP_NOP: break;
        case SQ_OP_FLIP_BOOLS: W(0); break;
        case SQ_OP_SWAP_BOOL_BOOL:
            W(0); W(1);
            if (in.imm[0] >= d.f[0].width || in.imm[1] >= d.f[1].width) fail(SQ_ERR_INVALID, "Swap_Bool_Bool: digit out of range");
            break;
        case SQ_OP_SHIFT_LEFT:
        case SQ_OP_SHIFT_RIGHT:
            W(0);
            if (in.imm[0] > d.f[0].width) fail(SQ_ERR_INVALID, "Shift: digit > register size");
            break;
        case SQ_OP_MULT_UINT_CONST:
        case SQ_OP_ADD_MULT_UINT_CONST:
            R(0); W(2);
            distinct(in.reg[0], in.reg[2], "Mult/Add_Mult");
            break;
        case SQ_OP_MOD_MULT_CONST:
            W(0);
            if (in.imm[1] == 0) fail(SQ_ERR_INVALID, "Mod_Mult: N == 0");
            break;
        case SQ_OP_ADD_UINT_UINT:
        case SQ_OP_SUB_UINT_UINT:
        case SQ_OP_MUL_UINT_UINT:
        case SQ_OP_DIV_UINT_UINT:
        case SQ_OP_AND_UINT_UINT:
        case SQ_OP_OR_UINT_UINT:
        case SQ_OP_XOR_UINT_UINT:
        case SQ_OP_LESS_SINT_SINT:
        case SQ_OP_LESS_UINT_UINT:
        case SQ_OP_GETMID_UINT_UINT:
            R(0); R(1); W(2);
            distinct(in.reg[0], in.reg[2], "out-of-place arithmetic");
            distinct(in.reg[1], in.reg[2], "out-of-place arithmetic");
            break;
        case SQ_OP_ADD_UINT_UINT_INPLACE:
            R(0); W(1);
            distinct(in.reg[0], in.reg[1], "Add_UInt_UInt_InPlace");
            break;
        case SQ_OP_ADD_UINT_CONST: R(0); W(2); distinct(in.reg[0], in.reg[2], "Add_UInt_ConstUInt"); break;
        case SQ_OP_ADD_CONST_INPLACE: W(0); break;
        case SQ_OP_PLUS_ONE_OVERFLOW:
            W(0); W(1);
            distinct(in.reg[0], in.reg[1], "PlusOneAndOverflow");
            break;
        case SQ_OP_BIT_GATHER:
            W(0);
            if (d.f[0].width < 64 && (in.imm[0] >> d.f[0].width)) fail(SQ_ERR_INVALID, "bit gather: position >= register size");
            break;
        case SQ_OP_NEG_UINT:
        case SQ_OP_ABS_SINT:
        case SQ_OP_SQRT_UINT:
        case SQ_OP_ISZERO_UINT:
        case SQ_OP_NEGATIVE_SINT:
            R(0); W(1);
            distinct(in.reg[0], in.reg[1], "unary arithmetic");
            break;
        case SQ_OP_SELECT_BOOL: R(0); R(1); R(2); W(3); break;
        case SQ_OP_CARRY_UINT_UINT:
        case SQ_OP_OVERFLOW_SINT_SINT:
        case SQ_OP_MULOVERFLOW_UINT_UINT:
            R(0); R(1); F(2); W(3);
            if (in.op == SQ_OP_OVERFLOW_SINT_SINT && d.f[2].width == 0) fail(SQ_ERR_INVALID, "Overflow: zero width");
            break;
        case SQ_OP_ADD_ANYINT_INPLACE: W(0); R(1); distinct(in.reg[0], in.reg[1], "Add_AnyInt_AnyInt_InPlace"); break;
        case SQ_OP_ASSIGN: R(0); W(1); break;
        case SQ_OP_COMPARE_UINT_UINT: R(0); R(1); W(2); W(3); break;
        case SQ_OP_SWAP_GENERAL: W(0); W(1); break;
        case SQ_OP_X_BOOL:
        case SQ_OP_Y_BOOL:
            W(0);
            if (in.imm[0] >= d.f[0].width) fail(SQ_ERR_INVALID, "gate digit >= register size");
            if (in.op == SQ_OP_Y_BOOL) am |= 3u;
            break;
        case SQ_OP_INIT_UNSAFE: W(0); break;
        case SQ_OP_QRAM_LOAD: {
            R(0); W(1);
            distinct(in.reg[0], in.reg[1], "QRAMLoad");
            const QramTable* q = reinterpret_cast<const QramTable*>(in.qram);
            if (!q || !q->dev) fail(SQ_ERR_INVALID, "QRAMLoad: null table");
            if (q->lookup || q->pair_kind >= 0) fail(SQ_ERR_INVALID, "QRAMLoad: not a QRAM table");
            if (d.f[1].width < 64 && q->max_word > wmask(d.f[1].width))
                fail(SQ_ERR_INVALID, "QRAMLoad: table word wider than the data register");
            d.table = q->dev;
            replay_note_input(q->dev, q->n_words * q->elem_bytes);
            d.elem_bytes = q->elem_bytes;
            d.addr_bits = q->address_size;
            break;
        }
        case SQ_OP_PHASE_BOOL:
            R(0);
            if (in.imm[0] >= d.f[0].width) fail(SQ_ERR_INVALID, "Phase_Bool: digit >= register size");
            am |= 3u;
            break;
        case SQ_OP_GLOBAL_PHASE: am |= 3u; break;
        case SQ_OP_REFLECTION_BOOL:
        case SQ_OP_ZERO_COND_PHASE_FLIP:
            for (uint32_t id = 0; id < 64; ++id) {
                if (!((in.imm[0] >> id) & 1ull)) continue;
                Field f = t.field(id);
                if (f.width) {
                    d.zmask[f.word] |= wmask(f.width) << f.shift;
                    rw |= 1u << f.word;
                }
            }
            am |= 3u;
            break;
        case SQ_OP_ROT_DIAGONAL:
            R(0);
            if (in.imm[0] >= d.f[0].width) fail(SQ_ERR_INVALID, "Rot_Bool: digit >= register size");
            am |= 3u;
            break;
        case SQ_OP_ROT_OFF_DIAGONAL:
            W(0);
            if (in.imm[0] >= d.f[0].width) fail(SQ_ERR_INVALID, "Rot_Bool: digit >= register size");
            am |= 3u;
            break;
        case SQ_OP_TRIDIAG_ELEMENT:
        case SQ_OP_TRIDIAG_SLOT_COLUMN: {
            const bool el = in.op == SQ_OP_TRIDIAG_ELEMENT;
            const char* what = el ? "TridiagOracle1" : "TridiagOracle2";
            R(0); R(1);
            if (el) { R(2); W(3); } else { W(2); W(3); }
            for (int x = 0; x < 3; ++x)
                for (int y = x + 1; y < 4; ++y)
                    if (el ? y == 3 : y >= 2) distinct(in.reg[x], in.reg[y], what);
            const uint64_t n = in.imm[0];
            if (n < 8 || (n & (n - 1))) fail(SQ_ERR_INVALID, std::string(what) + ": n must be a power of two >= 8");
            if (!el && (in.imm[2] == 0 || in.imm[2] > 64)) fail(SQ_ERR_INVALID, "TridiagOracle2: k_width out of range");
            break;
        }
        case SQ_OP_LOOKUP_XOR: {
            R(0); W(1);
            distinct(in.reg[0], in.reg[1], "lookup");
            const QramTable* q = reinterpret_cast<const QramTable*>(in.qram);
            if (!q || !q->dev || !q->lookup) fail(SQ_ERR_INVALID, "lookup: not a table of sq_lookup_create");
            if (d.f[1].width < 64 && q->max_word > wmask(d.f[1].width))
                fail(SQ_ERR_INVALID, "lookup: table word wider than the output register");
            d.table = q->dev;
            d.imm[0] = q->dense_len;
            d.imm[1] = q->n_sparse;
            replay_note_input(q->dev, q->n_words * 8);
            break;
        }
        case SQ_OP_PARITY_PHASE: R(0); am |= 3u; break;
        case SQ_OP_ADDR_XOR:
            R(0); R(1);
            if (in.imm[1]) R(2);
            W(3);
            distinct(in.reg[0], in.reg[3], "GetRowAddr/GetDataAddr");
            distinct(in.reg[1], in.reg[3], "GetRowAddr/GetDataAddr");
            if (in.imm[1]) distinct(in.reg[2], in.reg[3], "GetDataAddr");
            break;
        case SQ_OP_QBS_XOR: {
            R(0); R(1); W(2);
            distinct(in.reg[0], in.reg[2], "QuantumBinarySearch_Fast");
            distinct(in.reg[1], in.reg[2], "QuantumBinarySearch_Fast");
            const QramTable* q = reinterpret_cast<const QramTable*>(in.qram);
            if (!q || !q->dev) fail(SQ_ERR_INVALID, "QuantumBinarySearch_Fast: null table");
            if (q->lookup || q->pair_kind >= 0) fail(SQ_ERR_INVALID, "QuantumBinarySearch_Fast: not a QRAM table");
            if (in.imm[1] > 64) fail(SQ_ERR_INVALID, "QuantumBinarySearch_Fast: more than 64 rounds");
            d.table = q->dev;
            replay_note_input(q->dev, q->n_words * q->elem_bytes);
            d.elem_bytes = q->elem_bytes;
            d.addr_bits = q->address_size;
            break;
        }
        case SQ_OP_ANGLE_XOR: {
            R(0); R(1); W(2);
            distinct(in.reg[0], in.reg[2], "angle");
            distinct(in.reg[1], in.reg[2], "angle");
            const QramTable* q = reinterpret_cast<const QramTable*>(in.qram);
            if (!q || !q->dev || q->pair_kind < 0) fail(SQ_ERR_INVALID, "angle: not a table of sq_angle_table_create");
            if ((int)in.imm[0] != q->pair_kind) fail(SQ_ERR_INVALID, "angle: the table was made for the other operator");
            if (d.f[0].width != q->pair_w[0] || d.f[1].width != q->pair_w[1] || d.f[2].width != q->pair_w[2])
                fail(SQ_ERR_INVALID, "angle: the table was made for other register widths");
            d.table = q->dev;
            d.imm[0] = q->pair_mask;
            d.imm[1] = q->pair_probe;
            replay_note_input(q->dev, q->n_words * 8);
            break;
        }
        case SQ_OP_PAULI_NOISE: {
            R(0); W(1); W(2); W(3);
            const QramTable* q = reinterpret_cast<const QramTable*>(in.qram);
            if (!q || !q->dev) fail(SQ_ERR_INVALID, "Pauli noise: null mask table");
            if (q->n_words < 6 * in.imm[0]) fail(SQ_ERR_INVALID, "Pauli noise: table smaller than 6 words per trajectory");
            d.table = q->dev;
            replay_note_input(q->dev, q->n_words * q->elem_bytes);
            d.elem_bytes = q->elem_bytes;
            am |= 3u;
            break;
        }
        default: fail(SQ_ERR_INVALID, "unknown opcode " + std::to_string(in.op));
    }
    d.amask = wmask(d.addr_bits);
}

void run_program(State& s, const sq_instr* prog, uint32_t n) {
    if (n == 0) return;
    if (n > SQ_MAX_PROGRAM) fail(SQ_ERR_CAPACITY, "program longer than SQ_MAX_PROGRAM");
    uint32_t rw = 0, ww = 0, am = 0;
    uint32_t k = regtable().k;
    sync_words(s);
    if (s.n == 0) {
        // still validate arguments like the reference constructors would
        DInstr tmp;
        for (uint32_t i = 0; i < n; ++i) translate(prog[i], tmp, rw, ww, am);
        return;
    }
    if (n <= 4) {
        ProgramArgs<4> a;
        memset(&a, 0, sizeof(a));
        for (uint32_t i = 0; i < n; ++i) translate(prog[i], a.ins[i], rw, ww, am);
        a.err = device_error_word();
        a.n = n;
        a.read_words = rw;
        a.write_words = ww;
        a.amp_mode = am;
        if (ww) drop_groups(s);  // key values change: cached group ranges no longer hold
        dispatch_k<4>(a, s, k);
    } else {
        ProgramArgs<SQ_MAX_PROGRAM>* a = new ProgramArgs<SQ_MAX_PROGRAM>;
        memset(a, 0, sizeof(*a));
        try {
            for (uint32_t i = 0; i < n; ++i) translate(prog[i], a->ins[i], rw, ww, am);
        } catch (...) {
            delete a;
            throw;
        }
        a->err = device_error_word();
        a->n = n;
        a->read_words = rw;
        a->write_words = ww;
        a->amp_mode = am;
        if (ww) drop_groups(s);
        dispatch_k<SQ_MAX_PROGRAM>(*a, s, k);
        delete a;
    }
}

// QRAM tables are stored at the narrowest width that holds every word. The
// words are copied as they are, then narrowed on the GPU, which also ORs them
// together (the highest bit any word uses). dst == nullptr: the OR only.
__global__ void qram_pack_kernel(const uint64_t* __restrict__ src, uint64_t n, uint32_t eb, void* __restrict__ dst,
                                 unsigned long long* __restrict__ all) {
    const uint64_t stride = (uint64_t)gridDim.x * blockDim.x;
    unsigned long long acc = 0;
    for (uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += stride) {
        const uint64_t v = src[i];
        acc |= v;
        if (!dst) continue;
        if (eb == 2) ((unsigned short*)dst)[i] = (unsigned short)v;
        else if (eb == 4) ((unsigned int*)dst)[i] = (unsigned int)v;
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) acc |= __shfl_xor_sync(0xffffffffu, acc, o);
    if ((threadIdx.x & 31u) == 0 && acc) atomicOr(all, acc);
}

static uint32_t width_bytes(uint64_t all) { return all <= 0xffffull ? 2 : (all <= 0xffffffffull ? 4 : 8); }

// New words for an existing table, in place and at its stored width: its
// device address (held by queued or captured launches) does not change.
// Returns the OR of the new words. The words are checked against the stored
// width before the table is touched: when one does not fit, the table keeps
// its content (and the caller reports the error).
uint64_t qram_rewrite(QramTable& t, const uint64_t* host_words) {
    cudaStream_t st = stream();
    const uint64_t n = t.n_words;
    uint64_t* raw = t.elem_bytes == 8 ? static_cast<uint64_t*>(t.dev) : (uint64_t*)dev_alloc(n * 8);
    unsigned long long* all = (unsigned long long*)dev_alloc(8);
    copy_h2d_async(raw, host_words, n * 8);
    SQ_CUDA(cudaMemsetAsync(all, 0, 8, st));
    const bool narrow = t.elem_bytes != 8;  // 8-byte words fit whatever they are
    prof_begin("qram_pack");
    qram_pack_kernel<<<grid_for(n, 256), 256, 0, st>>>(raw, n, t.elem_bytes, narrow ? nullptr : t.dev, all);
    prof_end((double)n * 8);
    SQ_CUDA(cudaGetLastError());
    const uint64_t h = read_word_mapped(all);  // synchronises: the caller's buffer may go out of scope
    const uint64_t fits = t.elem_bytes == 2 ? 0xffffull : t.elem_bytes == 4 ? 0xffffffffull : ~0ull;
    if (narrow && !(h & ~fits)) {
        SQ_CUDA(cudaMemsetAsync(all, 0, 8, st));
        prof_begin("qram_pack");
        qram_pack_kernel<<<grid_for(n, 256), 256, 0, st>>>(raw, n, t.elem_bytes, t.dev, all);
        prof_end((double)n * (8 + t.elem_bytes));
        SQ_CUDA(cudaGetLastError());
    }
    if (raw != t.dev) dev_free(raw);  // stream-ordered: after the pack
    dev_free(all);
    return h;
}

void* qram_upload(const uint64_t* host_words, uint64_t n, uint32_t eb_guess, uint32_t* eb_out, uint64_t* all_out) {
    cudaStream_t st = stream();
    uint64_t* raw = (uint64_t*)dev_alloc(n * 8);
    unsigned long long* all = (unsigned long long*)dev_alloc(8);
    void* dst = eb_guess == 8 ? (void*)raw : dev_alloc(n * eb_guess);
    SQ_CUDA(cudaMemcpyAsync(raw, host_words, n * 8, cudaMemcpyHostToDevice, st));
    SQ_CUDA(cudaMemsetAsync(all, 0, 8, st));
    prof_begin("qram_pack");
    qram_pack_kernel<<<grid_for(n, 256), 256, 0, st>>>(raw, n, eb_guess, dst, all);
    prof_end((double)n * (8 + (eb_guess == 8 ? 0 : eb_guess)));
    SQ_CUDA(cudaGetLastError());
    unsigned long long h = 0;
    SQ_CUDA(cudaMemcpyAsync(&h, all, 8, cudaMemcpyDeviceToHost, st));
    SQ_CUDA(cudaStreamSynchronize(st));  // the caller's buffer may be pinned: the copy is complete on return
    const uint32_t eb = width_bytes(h);
    if (eb != eb_guess) {  // the words need another width: narrow again from the raw copy
        if (dst != raw) dev_free(dst);
        dst = eb == 8 ? (void*)raw : dev_alloc(n * eb);
        if (eb != 8) {
            prof_begin("qram_pack");
            qram_pack_kernel<<<grid_for(n, 256), 256, 0, st>>>(raw, n, eb, dst, all);
            prof_end((double)n * (8 + eb));
            SQ_CUDA(cudaGetLastError());
        }
    }
    if (dst != raw) dev_free(raw);
    dev_free(all);
    *eb_out = eb;
    *all_out = h;
    return dst;
}

// Zero one register field in every entry (AddRegister on reused bits,
// remove_register_synchronous).
template <int K>
__global__ void zero_field_kernel(uint64_t* __restrict__ w, uint64_t keep_mask, uint64_t n) {
    const uint64_t stride = (uint64_t)gridDim.x * blockDim.x;
    for (uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += stride) w[i] &= keep_mask;
}

void zero_field(State& s, Field f) {
    drop_groups(s);
    sync_words(s);
    if (s.n == 0 || f.width == 0) return;
    const uint64_t keep = ~(wmask(f.width) << f.shift);
    prof_begin("zero_field");
    zero_field_kernel<1><<<grid_for(s.n, 256), 256, 0, stream()>>>(s.live.keys[f.word], keep, s.n);
    prof_end((double)s.n * 16);
    SQ_CUDA(cudaGetLastError());
}

// CombineRegister when the two fields are not adjacent: dst = first << |second| | second,
// old fields cleared.
template <int K>
__global__ void move_field_kernel(KeyPtrs keys, Field first, Field second, Field dst, uint64_t n) {
    const uint64_t stride = (uint64_t)gridDim.x * blockDim.x;
    for (uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += stride) {
        uint64_t k[K];
#pragma unroll
        for (int w = 0; w < K; ++w) k[w] = keys.w[w][i];
        const uint64_t a = fget<K>(k, first), b = fget<K>(k, second);
        const uint64_t v = second.width >= 64 ? b : ((a << second.width) | b);
        fset<K>(k, first, 0);
        fset<K>(k, second, 0);
        fset<K>(k, dst, v);
#pragma unroll
        for (int w = 0; w < K; ++w) keys.w[w][i] = k[w];
    }
}

void move_field(State& s, Field first, Field second, Field dst) {
    drop_groups(s);
    sync_words(s);
    if (s.n == 0) return;
    KeyPtrs kp;
    for (int w = 0; w < SQ_KMAX; ++w) kp.w[w] = s.live.keys[w];
    unsigned g = grid_for(s.n, 256);
    prof_begin("move_field");
    switch (regtable().k) {
        case 1: move_field_kernel<1><<<g, 256, 0, stream()>>>(kp, first, second, dst, s.n); break;
        case 2: move_field_kernel<2><<<g, 256, 0, stream()>>>(kp, first, second, dst, s.n); break;
        case 3: move_field_kernel<3><<<g, 256, 0, stream()>>>(kp, first, second, dst, s.n); break;
        case 4: move_field_kernel<4><<<g, 256, 0, stream()>>>(kp, first, second, dst, s.n); break;
        case 5: move_field_kernel<5><<<g, 256, 0, stream()>>>(kp, first, second, dst, s.n); break;
        case 6: move_field_kernel<6><<<g, 256, 0, stream()>>>(kp, first, second, dst, s.n); break;
        case 7: move_field_kernel<7><<<g, 256, 0, stream()>>>(kp, first, second, dst, s.n); break;
        default: move_field_kernel<8><<<g, 256, 0, stream()>>>(kp, first, second, dst, s.n); break;
    }
    prof_end((double)s.n * 16.0 * regtable().k);
    SQ_CUDA(cudaGetLastError());
}

}  // namespace sq
