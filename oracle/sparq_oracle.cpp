// sparq_oracle.cpp — TEST INFRASTRUCTURE ONLY. A CPU restatement of SparQ's
// CPU operator path (the reference's std::vector<System> overloads), used by
// tests/, __graft_entry__.smoke() and bench.py's cpu_baseline leg as the
// checker. Nothing in the shipped engine links or calls this file.
//
// Representation mirrors the reference exactly: one entry ("System") is a
// complex<double> amplitude plus one uint64 word per register id
// (basic_components.h:221-297); the register table is process-global
// (basic_components.h:239-271). Every operator restates the reference's CPU
// algorithm step for step — sort/bucket order, the arithmetic order of every
// amplitude update, and the ClearZero that follows split operators — so that
// keys match bit for bit and amplitudes match to the last ulp where the
// reference is deterministic.
//
// The reference's helper library (git submodule extern/qram-simulator) is
// absent, so these helpers are restated from their observable semantics:
//   width_mask(w)   low-w-bit mask, all ones for w >= 64
//                   (spelled out at quantum_arithmetic.cpp:332)
//   get_complement  two's-complement value of a w-bit field
//   epsilon         1e-14 (clearzero_default_eps; documented in the reference's
//                   verification notes, not in code: unpinned constant)
//   sqrt2inv        correctly rounded 1/sqrt(2) (unpinned constant)
//   pi              M_PI
//   sort_merge_unique_erase  sort by System::operator<, sum runs of equal keys
//                   into the first, erase |a|^2 < epsilon (summation order
//                   within a run is parity-unpinned)
//
// Built with -ffp-contract=off so that no multiply-add is fused, on x86 and on
// aarch64 alike.
#include <algorithm>
#include <cmath>
#include <complex>
#include <cstdint>
#include <cstring>
#include <map>
#include <set>
#include <numeric>
#include <stdexcept>
#include <string>
#include <limits>
#include <vector>

#include "sparq_gb300.h"

namespace sqo {

using complex_t = std::complex<double>;

static const double kEpsilon = 1e-14;
static const double kSqrt2Inv = 1.0 / std::sqrt(2.0);
static const double kPi = 3.14159265358979323846;
static double g_clearzero_eps = kEpsilon;

struct RegInfo {
    uint32_t type;
    size_t size;
    bool active;
};
static std::vector<RegInfo> g_regs;          // System::name_register_map
static std::vector<size_t> g_reusable;       // System::reusable_registers
static std::string g_err;

struct System {
    complex_t amplitude{1.0, 0.0};
    mutable std::vector<uint64_t> registers;
    uint64_t& get(size_t id) {
        if (registers.size() < g_regs.size()) registers.resize(g_regs.size(), 0);
        return registers[id];
    }
    uint64_t get(size_t id) const {
        if (registers.size() < g_regs.size()) registers.resize(g_regs.size(), 0);
        return registers[id];
    }
};
using State = std::vector<System>;

static inline uint64_t pow2(size_t n) { return n >= 64 ? 0 : (uint64_t{1} << n); }
static inline uint64_t width_mask(size_t w) { return w >= 64 ? ~uint64_t{0} : pow2(w) - 1; }
static inline size_t size_of(size_t id) { return g_regs.at(id).size; }
static inline bool status_of(size_t id) { return g_regs.at(id).active; }
// StateStorage::as<uint64_t> (basic_components.h:102-131)
static inline uint64_t as_u64(uint64_t value, size_t size) {
    uint64_t m = size >= 64 ? ~uint64_t{0} : pow2(size) - (size != 0);
    return value & m;
}
static inline uint64_t get_as(const System& s, size_t id) { return as_u64(s.get(id), size_of(id)); }
static inline int64_t get_complement(uint64_t v, size_t size) {
    if (size == 0) return 0;
    if (size >= 64) return (int64_t)v;
    if ((v >> (size - 1)) & 1) return (int64_t)(v - pow2(size));
    return (int64_t)v;
}
static inline double as_double(uint64_t value, size_t size) {
    uint64_t t = as_u64(value, size);
    if (size == 64) return t * 1.0 / 2 / pow2(63);
    return 1.0 * t / (double)pow2(size);
}
static inline double abs_sqr(const complex_t& a) { return a.real() * a.real() + a.imag() * a.imag(); }
// complex * complex exactly as the straightforward formula (what GCC emits for
// finite operands; fused multiply-add disabled at build time).
static inline complex_t cmul(const complex_t& a, const complex_t& b) {
    return complex_t(a.real() * b.real() - a.imag() * b.imag(), a.real() * b.imag() + a.imag() * b.real());
}
static inline complex_t cscale(const complex_t& a, double s) { return complex_t(a.real() * s, a.imag() * s); }
static inline int bitcount(uint64_t v) { return __builtin_popcountll(v); }

// ---------------------------------------------------------------- conditions
// ConditionSatisfied (global_macros.h:28-86)
static bool condition_satisfied(const System& s, const sq_cond* c) {
    if (!c) return true;
    for (uint32_t i = 0; i < c->count; ++i) {
        const sq_condition& q = c->c[i];
        uint64_t raw = s.get(q.reg);
        size_t sz = size_of(q.reg);
        switch (q.kind) {
            case SQ_COND_NONZERO: if (!as_u64(raw, sz)) return false; break;
            case SQ_COND_ALL_ONES: if (raw != width_mask(sz)) return false; break;
            case SQ_COND_BIT: if (!(raw & pow2(q.param))) return false; break;
            case SQ_COND_VALUE: if (raw != q.param) return false; break;
            default: throw std::invalid_argument("bad condition kind");
        }
    }
    return true;
}

static void clear_zero(State& st, double eps) {
    // ClearZero::operator() (system_operations.cpp:371-382)
    auto it = std::remove_if(st.begin(), st.end(), [eps](const System& s) { return abs_sqr(s.amplitude) < eps; });
    st.erase(it, st.end());
}

static uint64_t isqrt_u64(uint64_t v) {
    // floor(sqrt(v)), bit-by-bit (the reference documents a pure integer
    // isqrt, quantum_arithmetic.h:1720-1722)
    uint64_t res = 0, bit = uint64_t{1} << 62;
    while (bit > v) bit >>= 2;
    while (bit) {
        if (v >= res + bit) { v -= res + bit; res = (res >> 1) + bit; }
        else res >>= 1;
        bit >>= 2;
    }
    return res;
}

struct Qram {
    uint32_t address_size;
    uint32_t data_size;
    std::vector<uint64_t> memory;
};

// ---------------------------------------------------------------- tridiagonal CKS oracles
// TridiagonalSpec (SparQ_Algorithm/include/hamiltonian_simulation_tridiagonal.h:
// 104-190): row j's 4-slot window starts at clamp(j - 1, 0, n - 4); the
// combined table word at idx & (8n - 1) is the quantised element of (row,
// slot) in the first half and the window column in the second.
static uint64_t tri_window_base(uint64_t j, uint64_t n) {
    uint64_t b = (j > 0) ? (j - 1) : 0;
    uint64_t bmax = n - 4;
    return b < bmax ? b : bmax;
}
static uint64_t tri_value_of(uint64_t j, uint64_t s, uint64_t n, uint64_t alpha_enc, uint64_t beta_enc) {
    uint64_t c = tri_window_base(j, n) + s;
    if (c == j) return alpha_enc;
    if (c + 1 == j || c == j + 1) return beta_enc;
    return 0;
}
static uint64_t tri_combined_mem(uint64_t idx, uint64_t n, uint64_t alpha_enc, uint64_t beta_enc) {
    idx &= 8 * n - 1;
    uint64_t half = n * 4;
    if (idx < half) return tri_value_of(idx >> 2, idx & 3, n, alpha_enc, beta_enc);
    uint64_t t = idx - half;
    return tri_window_base(t >> 2, n) + (t & 3);
}

// GetQWRotateAngle_Int_Int_Int (SparQ_Algorithm/src/hamiltonian_simulation.cpp:
// 257-291): the Rational fixed point of acos(sqrt(ratio)) / pi / 2, XORed
// into the output register; get_rational truncates (value * 2^size).
static uint64_t qw_rational(double x, size_t size) { return (uint64_t)(x * (double)pow2(size)); }
static void qw_rotate_angle(State& st, uint32_t data, uint32_t out, uint32_t data_size, bool positive_only,
                            const sq_cond* cond) {
    for (auto& s : st) {
        if (!condition_satisfied(s, cond)) continue;
        uint64_t v = get_as(s, data);
        double ratio;
        if (positive_only) {
            uint64_t amax = pow2(data_size) - 1;
            v = v % (amax + 1);
            ratio = v * 1.0 / amax;
        } else {
            uint64_t amax = pow2(data_size - 1) - 1;
            v = v % pow2(data_size);
            int64_t vr = get_complement(v, data_size);
            ratio = std::abs(vr) * 1.0 / amax;
        }
        ratio = std::max(0.0, std::min(1.0, ratio));
        double a = std::acos(std::sqrt(ratio)) / M_PI / 2;
        s.get(out) ^= qw_rational(a, size_of(out));
    }
}

// ---------------------------------------------------------------- elementwise
static void apply_instr_entry(System& s, const sq_instr& in) {
    const uint32_t* r = in.reg;
    switch (in.op) {
        case SQ_OP_NOP: return;
        case SQ_OP_FLIP_BOOLS: {  // quantum_arithmetic.cpp:11-30
            uint64_t& v = s.get(r[0]);
            v = (~v) & width_mask(size_of(r[0]));
            return;
        }
        case SQ_OP_SWAP_BOOL_BOOL: {  // :32-61
            uint64_t& a = s.get(r[0]);
            uint64_t& b = s.get(r[1]);
            bool v1 = (a >> in.imm[0]) & 1, v2 = (b >> in.imm[1]) & 1;
            if (v1 && !v2) { a -= pow2(in.imm[0]); b += pow2(in.imm[1]); }
            if (v2 && !v1) { a += pow2(in.imm[0]); b -= pow2(in.imm[1]); }
            return;
        }
        case SQ_OP_SHIFT_LEFT:
        case SQ_OP_SHIFT_RIGHT: {  // :63-135 (dag swaps direction)
            size_t size = size_of(r[0]);
            size_t digit = in.imm[0];
            bool left = (in.op == SQ_OP_SHIFT_LEFT) != (in.dag != 0);
            uint64_t value = get_as(s, r[0]);
            if (left) {
                uint64_t high = (size - digit) >= 64 ? 0 : value >> (size - digit);
                uint64_t low = value - ((size - digit) >= 64 ? 0 : (high << (size - digit)));
                s.get(r[0]) = (digit >= 64 ? 0 : (low << digit)) + high;
            } else {
                uint64_t high = digit >= 64 ? 0 : value >> digit;
                uint64_t low = value - (digit >= 64 ? 0 : (high << digit));
                s.get(r[0]) = ((size - digit) >= 64 ? 0 : (low << (size - digit))) + high;
            }
            return;
        }
        case SQ_OP_MULT_UINT_CONST: {  // :137-155
            uint64_t& o = s.get(r[2]);
            o = (o ^ (get_as(s, r[0]) * in.imm[0])) & width_mask(size_of(r[2]));
            return;
        }
        case SQ_OP_ADD_MULT_UINT_CONST: {  // :157-196
            uint64_t& o = s.get(r[2]);
            uint64_t m = width_mask(size_of(r[2]));
            if (!in.dag) o = (o + in.imm[0] * get_as(s, r[0])) & m;
            else o = (o - get_as(s, r[0]) * in.imm[0]) & m;
            return;
        }
        case SQ_OP_MOD_MULT_CONST: {  // :222-285 (imm0 = opnum or its inverse, imm1 = N)
            uint64_t v = get_as(s, r[0]);
            s.get(r[0]) = (v * in.imm[0]) % in.imm[1];
            return;
        }
        case SQ_OP_ADD_UINT_UINT: {  // :287-306
            uint64_t& o = s.get(r[2]);
            o = (o ^ (get_as(s, r[0]) + get_as(s, r[1]))) & width_mask(size_of(r[2]));
            return;
        }
        case SQ_OP_ADD_UINT_UINT_INPLACE: {  // :308-349
            uint64_t& o = s.get(r[1]);
            uint64_t m = width_mask(size_of(r[1]));
            if (!in.dag) o = (o + get_as(s, r[0])) & m;
            else o = (o - get_as(s, r[0])) & m;
            return;
        }
        case SQ_OP_ADD_UINT_CONST: {  // :351-369
            uint64_t& o = s.get(r[2]);
            o = (o ^ (get_as(s, r[0]) + in.imm[0])) & width_mask(size_of(r[2]));
            return;
        }
        case SQ_OP_ADD_CONST_INPLACE: {  // :371-411
            uint64_t& o = s.get(r[0]);
            uint64_t m = width_mask(size_of(r[0]));
            if (!in.dag) o = (o + in.imm[0]) & m;
            else o = (o - in.imm[0]) & m;
            return;
        }
        case SQ_OP_PLUS_ONE_OVERFLOW: {  // block_encoding_tridiagonal.cpp:20-83
            uint64_t& v = s.get(r[0]);
            uint64_t& ov = s.get(r[1]);
            const uint64_t top = width_mask(size_of(r[0]));
            if (!in.dag) {
                if (v == top) {
                    ov = (ov + 1) % 2;
                    v = 0;
                } else {
                    v += 1;
                }
            } else {
                if (v == 0) {
                    ov = (ov + 1) % 2;
                    v = top;
                } else {
                    v -= 1;
                }
            }
            return;
        }
        case SQ_OP_SUB_UINT_UINT: {  // :490-509
            uint64_t& o = s.get(r[2]);
            o = (o ^ (get_as(s, r[0]) - get_as(s, r[1]))) & width_mask(size_of(r[2]));
            return;
        }
        case SQ_OP_NEG_UINT: {  // :511-530
            uint64_t& o = s.get(r[1]);
            o = (o ^ (uint64_t{0} - get_as(s, r[0]))) & width_mask(size_of(r[1]));
            return;
        }
        case SQ_OP_ABS_SINT: {  // :532-554
            int64_t v = get_complement(get_as(s, r[0]), size_of(r[0]));
            uint64_t mag = v < 0 ? (uint64_t)(-v) : (uint64_t)v;
            uint64_t& o = s.get(r[1]);
            o = (o ^ mag) & width_mask(size_of(r[1]));
            return;
        }
        case SQ_OP_MUL_UINT_UINT: {  // :556-575
            uint64_t& o = s.get(r[2]);
            o = (o ^ (get_as(s, r[0]) * get_as(s, r[1]))) & width_mask(size_of(r[2]));
            return;
        }
        case SQ_OP_DIV_UINT_UINT: {  // :577-600
            uint64_t a = get_as(s, r[0]), b = get_as(s, r[1]);
            uint64_t q = b == 0 ? 0 : a / b;
            uint64_t& o = s.get(r[2]);
            o = (o ^ q) & width_mask(size_of(r[2]));
            return;
        }
        case SQ_OP_SQRT_UINT: {  // :602-620
            uint64_t& o = s.get(r[1]);
            o = (o ^ isqrt_u64(get_as(s, r[0]))) & width_mask(size_of(r[1]));
            return;
        }
        case SQ_OP_SELECT_BOOL: {  // :623-644
            uint64_t c = get_as(s, r[0]) & 1;
            uint64_t sel = c ? get_as(s, r[1]) : get_as(s, r[2]);
            uint64_t& o = s.get(r[3]);
            o = (o ^ sel) & width_mask(size_of(r[3]));
            return;
        }
        case SQ_OP_AND_UINT_UINT:
        case SQ_OP_OR_UINT_UINT:
        case SQ_OP_XOR_UINT_UINT: {  // :646-707
            uint64_t a = get_as(s, r[0]), b = get_as(s, r[1]);
            uint64_t v = in.op == SQ_OP_AND_UINT_UINT ? (a & b) : in.op == SQ_OP_OR_UINT_UINT ? (a | b) : (a ^ b);
            uint64_t& o = s.get(r[2]);
            o = (o ^ v) & width_mask(size_of(r[2]));
            return;
        }
        case SQ_OP_LESS_SINT_SINT: {  // :709-729
            int64_t l = get_complement(get_as(s, r[0]), size_of(r[0]));
            int64_t rr = get_complement(get_as(s, r[1]), size_of(r[1]));
            s.get(r[2]) ^= (l < rr) ? 1 : 0;
            return;
        }
        case SQ_OP_CARRY_UINT_UINT: {  // :731-754
            uint64_t a = get_as(s, r[0]), b = get_as(s, r[1]);
            size_t w = size_of(r[2]);
            bool pred = w >= 64 ? (a + b < a) : (a >= (uint64_t{1} << w)) || (b >= (uint64_t{1} << w) - a);
            s.get(r[3]) ^= pred ? 1 : 0;
            return;
        }
        case SQ_OP_OVERFLOW_SINT_SINT: {  // :756-785
            size_t w = size_of(r[2]);
            uint64_t m = width_mask(w);
            uint64_t A = (uint64_t)get_complement(get_as(s, r[0]), size_of(r[0])) & m;
            uint64_t B = (uint64_t)get_complement(get_as(s, r[1]), size_of(r[1])) & m;
            uint64_t S = (A + B) & m;
            uint64_t sa = (A >> (w - 1)) & 1, sb = (B >> (w - 1)) & 1, ss = (S >> (w - 1)) & 1;
            bool pred = (sa == sb) && (ss != sa);
            s.get(r[3]) ^= pred ? 1 : 0;
            return;
        }
        case SQ_OP_MULOVERFLOW_UINT_UINT: {  // :787-817
            uint64_t a = get_as(s, r[0]), b = get_as(s, r[1]);
            uint64_t lo = a * b;
            uint64_t hi = (uint64_t)(((unsigned __int128)a * (unsigned __int128)b) >> 64);
            size_t w = size_of(r[2]);
            bool pred = hi != 0 || (w < 64 && lo >= (uint64_t{1} << w));
            s.get(r[3]) ^= pred ? 1 : 0;
            return;
        }
        case SQ_OP_ISZERO_UINT: {  // :819-837
            s.get(r[1]) ^= (get_as(s, r[0]) == 0) ? 1 : 0;
            return;
        }
        case SQ_OP_NEGATIVE_SINT: {  // :839-857
            s.get(r[1]) ^= (get_complement(get_as(s, r[0]), size_of(r[0])) < 0) ? 1 : 0;
            return;
        }
        case SQ_OP_ADD_ANYINT_INPLACE: {  // :860-907
            size_t rsz = size_of(r[1]);
            uint64_t raw = get_as(s, r[1]);
            uint64_t ext = g_regs[r[1]].type == SQ_SIGNED ? (uint64_t)get_complement(raw, rsz) : raw;
            uint64_t& o = s.get(r[0]);
            uint64_t m = width_mask(size_of(r[0]));
            if (!in.dag) o = (o + ext) & m;
            else o = (o - ext) & m;
            return;
        }
        case SQ_OP_ASSIGN: {  // :909-930
            uint64_t& o = s.get(r[1]);
            o = (o ^ s.get(r[0])) & width_mask(size_of(r[1]));
            return;
        }
        case SQ_OP_COMPARE_UINT_UINT: {  // :932-959
            uint64_t l = get_as(s, r[0]), rr = get_as(s, r[1]);
            if (l == rr) s.get(r[3]) ^= 1;
            else s.get(r[2]) ^= (l < rr) ? 1 : 0;
            return;
        }
        case SQ_OP_LESS_UINT_UINT: {  // :961-980
            s.get(r[2]) ^= (get_as(s, r[0]) < get_as(s, r[1])) ? 1 : 0;
            return;
        }
        case SQ_OP_SWAP_GENERAL: {  // :982-999
            std::swap(s.get(r[0]), s.get(r[1]));
            return;
        }
        case SQ_OP_GETMID_UINT_UINT: {  // :1001-1020
            s.get(r[2]) ^= (get_as(s, r[0]) + get_as(s, r[1])) / 2;
            return;
        }
        case SQ_OP_X_BOOL: {  // basic_gates.cpp:383-401
            s.get(r[0]) ^= pow2(in.imm[0]);
            return;
        }
        case SQ_OP_INIT_UNSAFE: {  // dark_magic.cpp:35-40
            s.get(r[0]) = in.imm[0];
            return;
        }
        case SQ_OP_QRAM_LOAD: {  // qram.cpp:15-35
            const Qram* q = reinterpret_cast<const Qram*>(in.qram);
            uint64_t addr = get_as(s, r[0]) % pow2(q->address_size);
            s.get(r[1]) ^= q->memory[addr];
            return;
        }
        case SQ_OP_ADDR_XOR: {  // GetRowAddr / GetDataAddr (hamiltonian_simulation.cpp:222-253)
            // the reference XORs the whole sum in; a register here holds its width
            uint64_t v = get_as(s, r[0]) + in.imm[0] * get_as(s, r[1]);
            if (in.imm[1]) v += get_as(s, r[2]);
            s.get(r[3]) = (s.get(r[3]) ^ v) & width_mask(size_of(r[3]));
            return;
        }
        case SQ_OP_QBS_XOR: {  // QuantumBinarySearch_Fast (hamiltonian_simulation.cpp:182-220)
            const Qram* q = reinterpret_cast<const Qram*>(in.qram);
            const uint64_t target = get_as(s, r[1]);
            uint64_t l = get_as(s, r[0]), rr = l + in.imm[0], found = 0;
            for (uint64_t i = 0; i < in.imm[1]; ++i) {
                const uint64_t mid = (l + rr) / 2;
                const uint64_t word = q->memory[mid % pow2(q->address_size)];
                if (word == target) {
                    found = mid;
                    break;
                }
                if (word < target) l = mid;
                else rr = mid;
            }
            s.get(r[2]) = (s.get(r[2]) ^ found) & width_mask(size_of(r[2]));
            return;
        }
        case SQ_OP_PHASE_BOOL: {  // basic_gates.cpp:11-54 (c0 precomputed, conj for dag)
            if ((s.get(r[0]) >> in.imm[0]) & 1) s.amplitude = cmul(s.amplitude, complex_t(in.c[0], in.c[1]));
            return;
        }
        case SQ_OP_GLOBAL_PHASE: {  // parallel_phase_operations.cpp:72-107
            s.amplitude = cmul(s.amplitude, complex_t(in.c[0], in.c[1]));
            return;
        }
        case SQ_OP_Y_BOOL: {  // basic_gates.cpp:418-441
            uint64_t& v = s.get(r[0]);
            v ^= pow2(in.imm[0]);
            if ((v >> in.imm[0]) & 1) s.amplitude = cmul(s.amplitude, complex_t(0, 1));
            else s.amplitude = cmul(s.amplitude, complex_t(0, -1));
            return;
        }
        case SQ_OP_REFLECTION_BOOL: {  // parallel_phase_operations.cpp:46-70 (imm0 = register-id bitmask, imm1 = inverse)
            bool iszero = true;
            for (size_t id = 0; id < 64; ++id)
                if ((in.imm[0] >> id) & 1) iszero = iszero && (get_as(s, id) == 0);
            bool inverse = in.imm[1] != 0;
            if (!(inverse ^ iszero)) s.amplitude = complex_t(s.amplitude.real() * -1.0, s.amplitude.imag() * -1.0);
            return;
        }
        case SQ_OP_ZERO_COND_PHASE_FLIP: {  // parallel_phase_operations.cpp:11-31
            bool all = true;
            for (size_t id = 0; id < 64; ++id)
                if ((in.imm[0] >> id) & 1) all = all && (s.get(id) == 0);
            if (all) s.amplitude = complex_t(s.amplitude.real() * -1.0, s.amplitude.imag() * -1.0);
            return;
        }
        case SQ_OP_ROT_DIAGONAL: {  // basic_gates.cpp:110-133 (mask = bit imm0)
            if (s.get(r[0]) & pow2(in.imm[0])) s.amplitude = cmul(s.amplitude, complex_t(in.c[2], in.c[3]));
            else s.amplitude = cmul(s.amplitude, complex_t(in.c[0], in.c[1]));
            return;
        }
        case SQ_OP_ROT_OFF_DIAGONAL: {  // basic_gates.cpp:146-171; c0 = mat[2] (was 0), c1 = mat[1] (was 1)
            uint64_t& v = s.get(r[0]);
            if (v & pow2(in.imm[0])) s.amplitude = cmul(s.amplitude, complex_t(in.c[2], in.c[3]));
            else s.amplitude = cmul(s.amplitude, complex_t(in.c[0], in.c[1]));
            v ^= pow2(in.imm[0]);
            return;
        }
        case SQ_OP_TRIDIAG_ELEMENT: {  // TridiagOracle1, hamiltonian_tridiagonal.cpp:16-33
            uint64_t off = get_as(s, r[0]), j = get_as(s, r[1]), slot = get_as(s, r[2]);
            s.get(r[3]) ^= tri_combined_mem(off + 4 * j + slot, in.imm[0], in.imm[1] & 0xffffffffull,
                                            in.imm[1] >> 32);
            return;
        }
        case SQ_OP_TRIDIAG_SLOT_COLUMN: {  // TridiagOracle2, hamiltonian_tridiagonal.cpp:35-83
            const uint64_t n = in.imm[0], ae = in.imm[1] & 0xffffffffull, be = in.imm[1] >> 32;
            const uint64_t kmask = in.imm[2] >= 64 ? ~uint64_t{0} : pow2(in.imm[2]) - 1;
            uint64_t j = get_as(s, r[1]), off = get_as(s, r[0]), k = get_as(s, r[2]);
            uint64_t sr = get_as(s, r[3]) & kmask;  // the tag register, read at k_width bits
            uint64_t base = tri_window_base(j, n);
            uint64_t row_addr = off + 4 * j;
            if (!in.dag) {
                bool hit = k >= base && k < base + 4;
                uint64_t sr1 = sr ^ (hit ? row_addr + (k - base) : 0);
                uint64_t k1 = k ^ tri_combined_mem(sr1, n, ae, be);
                s.get(r[2]) = (sr1 - row_addr) & kmask;
                s.get(r[3]) = k1 & kmask;
            } else {
                uint64_t k1 = (k + row_addr) & kmask;
                uint64_t k2 = sr ^ tri_combined_mem(k1, n, ae, be);
                bool hit = k2 >= base && k2 < base + 4;
                s.get(r[2]) = k2;
                s.get(r[3]) = k1 ^ (hit ? row_addr + (k2 - base) : 0);
            }
            return;
        }
        case SQ_OP_ANGLE_XOR: {
            // imm0 = 0: Div_Sqrt_Arccos_UInt_UInt (quantum_arithmetic.cpp:413-432)
            //   out = acos(sqrt(1.0 * lhs / rhs)) / pi / 2 of the unsigned values;
            // imm0 = 1: GetRotateAngle_Int_Int (:458-487) of the two's-complement
            //   values: 0.25 / 0.75 for lhs = 0, else atan2(rhs, lhs) / pi / 2 in [0, 1).
            // regout ^= get_rational(out, size): truncation (a NaN angle gives 0;
            // the reference's conversion of NaN is undefined in C++).
            double out;
            if (in.imm[0] == 0) {
                uint64_t lv = get_as(s, r[0]), rv = get_as(s, r[1]);
                out = std::acos(std::sqrt(1.0 * lv / rv)) / kPi / 2;
            } else {
                int64_t l = get_complement(get_as(s, r[0]), size_of(r[0]));
                int64_t rr = get_complement(get_as(s, r[1]), size_of(r[1]));
                if (l == 0 && rr >= 0) out = 0.25;
                else if (l == 0 && rr < 0) out = 0.75;
                else {
                    out = std::atan2((double)rr, (double)l) / kPi / 2;
                    if (out < 0) out += 1;
                }
            }
            uint64_t word = std::isnan(out) ? 0 : (uint64_t)(out * (double)pow2(size_of(r[2])));
            s.get(r[2]) ^= word & width_mask(size_of(r[2]));
            return;
        }
        case SQ_OP_BIT_GATHER: {  // Hadamard_Partial's index map (hadamard.cpp:443-466)
            uint64_t& v = s.get(r[0]);
            const size_t w = size_of(r[0]);
            const uint64_t set = in.imm[0] & width_mask(w);
            std::vector<size_t> lo, hi;
            for (size_t b = 0; b < w; ++b) ((set >> b) & 1 ? lo : hi).push_back(b);
            lo.insert(lo.end(), hi.begin(), hi.end());  // new position k takes old bit lo[k]
            uint64_t out = 0;
            for (size_t k = 0; k < lo.size(); ++k) {
                if (in.dag) out |= ((v >> k) & 1ull) << lo[k];
                else out |= ((v >> lo[k]) & 1ull) << k;
            }
            v = out;
            return;
        }
        case SQ_OP_PARITY_PHASE: {  // TridiagParityPhase, hamiltonian_tridiagonal.cpp:88-105
            if (get_as(s, r[0]) & 1) s.amplitude = -s.amplitude;
            return;
        }
        case SQ_OP_PAULI_NOISE: {  // per-trajectory X then Z masks (batched trajectories)
            const Qram* q = reinterpret_cast<const Qram*>(in.qram);
            uint64_t t = get_as(s, r[0]);
            if (t >= in.imm[0]) return;
            int parity = 0;
            for (int k = 0; k < 3; ++k) {
                uint64_t& v = s.get(r[k + 1]);
                v ^= q->memory[t * 6 + k];
                parity += bitcount(v & q->memory[t * 6 + 3 + k]);
            }
            if (parity & 1) s.amplitude = complex_t(s.amplitude.real() * -1.0, s.amplitude.imag() * -1.0);
            return;
        }
        default:
            throw std::invalid_argument("unknown opcode " + std::to_string(in.op));
    }
}

static void apply_instr(State& st, const sq_instr& in) {
    for (auto& s : st) {
        if (!condition_satisfied(s, &in.cond)) continue;
        apply_instr_entry(s, in);
    }
}

// ---------------------------------------------------------------- grouping helpers
// SortExceptKey (sort_state.cpp:10-36)
static void sort_except_key(State& st, size_t id) {
    auto pred = [id](const System& l, const System& r) {
        for (size_t i = 0; i < g_regs.size(); ++i) {
            if (!status_of(i) || i == id) continue;
            uint64_t a = l.get(i), b = r.get(i);
            if (a < b) return true;
            if (a > b) return false;
        }
        return l.get(id) < r.get(id);
    };
    std::sort(st.begin(), st.end(), pred);
}
// compare_equal (sort_state.cpp:173-188)
static bool compare_equal(const System& a, const System& b, size_t out_id) {
    for (size_t i = g_regs.size(); i-- > 0;) {
        if (!status_of(i) || i == out_id) continue;
        if (a.get(i) != b.get(i)) return false;
    }
    return true;
}
// StateLessExceptKey (quantum_interfere_basic.cpp:130-149)
struct LessExceptKey {
    size_t id;
    bool operator()(const System& v1, const System& v2) const {
        for (size_t i = 0; i < g_regs.size(); ++i) {
            if (!status_of(i) || i == id) continue;
            uint64_t a = v1.get(i), b = v2.get(i);
            if (a < b) return true;
            if (a > b) return false;
        }
        return false;
    }
};

// ---------------------------------------------------------------- PartialTraceSelect
// partial_trace.cpp:148-225: remove_if (order kept) with the probability
// summed in order, then a *= 1/sqrt(p); returns that factor or +inf.
static double partial_trace_select(State& st, const std::vector<uint32_t>& regs,
                                   const std::vector<uint64_t>& values, bool range, uint64_t lo, uint64_t hi) {
    if (!range && regs.empty()) return 0;
    if (st.empty()) return 0;
    double sum_prob = 0;
    State kept;
    kept.reserve(st.size());
    for (const auto& s : st) {
        bool keep = true;
        if (range) {
            const uint64_t v = get_as(s, regs[0]);
            keep = v >= lo && v <= hi;
        } else {
            for (size_t i = 0; i < regs.size(); ++i)
                if (values[i] != s.get(regs[i])) {
                    keep = false;
                    break;
                }
        }
        if (keep) {
            sum_prob += abs_sqr(s.amplitude);
            kept.push_back(s);
        }
    }
    st.swap(kept);
    if (sum_prob != 0) {
        sum_prob = 1.0 / std::sqrt(sum_prob);
        for (auto& s : st) s.amplitude *= sum_prob;
        return sum_prob;
    }
    return std::numeric_limits<double>::infinity();
}

// ---------------------------------------------------------------- GetOutput
// GetOutput::operator() (SparQ_Algorithm qda_fundamental.cpp:123-166): the
// entries whose post-selected registers all hold 0 are written, in state
// order, to a dense vector at the concatenation of their index registers (the
// first in the lowest bits, qda_fundamental.h:640-645); sum = their total
// probability; the vector is scaled by 1/sqrt(sum) unless |sum - 1| < epsilon
// (a sum of 0 scales by 1).
static double get_output(const State& st, const std::vector<uint32_t>& zero, const std::vector<uint32_t>& idx,
                         std::vector<complex_t>& out) {
    size_t bits = 0;
    for (uint32_t r : idx) bits += size_of(r);
    out.assign(pow2(bits), complex_t(0, 0));
    double sum = 0.0;
    for (const auto& s : st) {
        bool is_zero = true;
        for (uint32_t r : zero)
            if (get_as(s, r) != 0) {
                is_zero = false;
                break;
            }
        if (!is_zero) continue;
        uint64_t id = 0;
        size_t off = 0;
        for (uint32_t r : idx) {
            id |= get_as(s, r) << off;
            off += size_of(r);
        }
        out[id] = s.amplitude;
        sum += abs_sqr(s.amplitude);
    }
    if (std::abs(sum - 1.0) < kEpsilon) return sum;
    const double k = sum != 0 ? 1.0 / std::sqrt(sum) : 1.0;
    for (auto& v : out) v *= k;
    return sum;
}

// ---------------------------------------------------------------- Hadamard_Int
// Hadamard_Int::operate (hadamard.cpp:18-132). Groups whose members disagree
// on the register's bits above n_digits make the reference write outside the
// state (its general case indexes val - value_mask); the restatement rejects
// them instead of reproducing undefined behaviour.
static void hadamard_int_operate(size_t l, size_t r, State& st, size_t id, size_t n_digits, uint64_t mask,
                                 const sq_cond* cond) {
    size_t n = r - l;
    size_t full_size = (size_t)pow2(n_digits);
    size_t original_size = st.size();
    double extra_amplitude = 1.0 / std::sqrt((double)full_size);
    if (n == 0) return;
    if (!condition_satisfied(st[l], cond)) return;
    for (size_t i = l + 1; i < r; ++i)
        if ((st[i].get(id) & mask) != (st[l].get(id) & mask))
            throw std::invalid_argument("Hadamard_Int: group members differ above n_digits (undefined in the reference)");
    if (n == 1) {
        uint64_t v = st[l].get(id);
        st[l].amplitude = cscale(st[l].amplitude, extra_amplitude);
        System base = st[l];
        st.insert(st.end(), full_size, base);
        for (size_t i = 0; i < full_size; ++i) {
            size_t pos = original_size + i;
            st[pos].get(id) = (st[pos].get(id) & mask) + i;
            if (bitcount(i & v) & 1) st[pos].amplitude = complex_t(st[pos].amplitude.real() * -1, st[pos].amplitude.imag() * -1);
        }
        st[l].amplitude = 0;
    } else if (n == full_size) {
        for (size_t qn = 0; qn < n_digits; ++qn)
            for (size_t i = 0; i < full_size; ++i)
                if ((i >> qn) & 1) {
                    complex_t a0 = st[i + l - pow2(qn)].amplitude, a1 = st[i + l].amplitude;
                    st[i + l - pow2(qn)].amplitude = cscale(a0 + a1, kSqrt2Inv);
                    st[i + l].amplitude = cscale(a0 - a1, kSqrt2Inv);
                }
    } else {
        System base = st[l];
        st.insert(st.end(), full_size, base);
        uint64_t value_mask = st[l].get(id) & mask;
        for (size_t i = 0; i < full_size; ++i) {
            st[i + original_size].amplitude = 0;
            st[i + original_size].get(id) = value_mask + i;
        }
        for (size_t i = l; i < r; ++i) {
            st[st[i].get(id) - value_mask + original_size].amplitude = st[i].amplitude;
            st[i].amplitude = 0;
        }
        for (size_t qn = 0; qn < n_digits; ++qn)
            for (size_t i = 0; i < full_size; ++i)
                if ((i >> qn) & 1) {
                    complex_t a0 = st[i + original_size - pow2(qn)].amplitude, a1 = st[i + original_size].amplitude;
                    st[i + original_size - pow2(qn)].amplitude = cscale(a0 + a1, kSqrt2Inv);
                    st[i + original_size].amplitude = cscale(a0 - a1, kSqrt2Inv);
                }
    }
}

// Hadamard_Int::operator() (hadamard.cpp:134-162)
static void hadamard_int(State& st, size_t id, size_t n_digits, const sq_cond* cond) {
    if (st.empty()) return;
    uint64_t mask = ~(pow2(n_digits) - 1);
    if (n_digits >= 64) mask = 0;
    sort_except_key(st, id);
    size_t current_size = st.size();
    size_t l = 0, r = 1;
    while (true) {
        if (r == current_size) { hadamard_int_operate(l, r, st, id, n_digits, mask, cond); break; }
        if (!compare_equal(st[l], st[r], id)) {
            hadamard_int_operate(l, r, st, id, n_digits, mask, cond);
            l = r;
            r = l + 1;
        } else {
            r++;
        }
    }
    clear_zero(st, g_clearzero_eps);
}

// ---------------------------------------------------------------- Hadamard_Int_Full
// hadamard.cpp:181-338 with SAFE_HASH (std::map buckets)
static void hadamard_full_inplace(const std::vector<size_t>& positions, State& st, size_t n_digits) {
    size_t full_size = (size_t)pow2(n_digits);
    std::vector<complex_t> amps(positions.size(), 0);
    for (size_t i = 0; i < positions.size(); ++i) amps[i] = st[positions[i]].amplitude;
    for (size_t qn = 0; qn < n_digits; ++qn)
        for (size_t i = 0; i < full_size; ++i)
            if ((i >> qn) & 1) {
                complex_t a0 = amps[i - pow2(qn)], a1 = amps[i];
                amps[i - pow2(qn)] = cscale(a0 + a1, kSqrt2Inv);
                amps[i] = cscale(a0 - a1, kSqrt2Inv);
            }
    for (size_t i = 0; i < positions.size(); ++i) st[positions[i]].amplitude = amps[i];
}

static void hadamard_full_sparse(const std::vector<size_t>& positions, State& st, size_t id, size_t n_digits) {
    size_t full_size = (size_t)pow2(n_digits);
    double extra_amplitude = 1.0 / std::sqrt((double)full_size);
    size_t original_size = st.size();
    bool inserted = false;
    for (size_t i = 0; i < positions.size(); ++i) {
        if (positions[i] == (size_t)-1) continue;
        uint64_t v = st[positions[i]].get(id);
        if (!inserted) {
            System base = st[positions[i]];
            st.insert(st.end(), full_size, base);
            for (size_t j = 0; j < full_size; ++j) {
                st[original_size + j].get(id) = j;
                st[original_size + j].amplitude = 0;
            }
            inserted = true;
        }
        for (size_t j = 0; j < full_size; ++j) {
            complex_t term = cscale(st[positions[i]].amplitude, (bitcount(j & v) & 1) ? -1. : 1.);
            term = cscale(term, extra_amplitude);
            st[original_size + j].amplitude += term;
        }
        st[positions[i]].amplitude = 0;
    }
}

static void hadamard_int_full(State& st, size_t id, const sq_cond* cond) {
    if (st.empty()) return;
    size_t n_digits = size_of(id);
    size_t full_size = (size_t)pow2(n_digits);
    size_t few_threshold = n_digits - 1;
    size_t current_size = st.size();
    std::map<System, std::pair<size_t, std::vector<size_t>>, LessExceptKey> buckets(LessExceptKey{id});
    for (size_t i = 0; i < current_size; ++i) {
        if (!condition_satisfied(st[i], cond)) continue;
        uint64_t val = get_as(st[i], id);
        auto res = buckets.insert({st[i], {0, std::vector<size_t>(full_size, (size_t)-1)}});
        auto iter = res.first;
        iter->second.second[val] = i;
        iter->second.first += 1;
        if (iter->second.first == full_size) {
            hadamard_full_inplace(iter->second.second, st, n_digits);
            buckets.erase(iter);
        }
    }
    for (auto& kv : buckets) {
        auto& all_pos = kv.second.second;
        if (kv.second.first <= few_threshold) {
            hadamard_full_sparse(all_pos, st, id, n_digits);
            continue;
        }
        for (size_t i = 0; i < all_pos.size(); ++i) {
            if (all_pos[i] == (size_t)-1) {
                st.push_back(kv.first);
                st.back().get(id) = i;
                st.back().amplitude = 0;
                all_pos[i] = st.size() - 1;
            }
        }
        hadamard_full_inplace(all_pos, st, n_digits);
    }
    clear_zero(st, g_clearzero_eps);
}

// ---------------------------------------------------------------- Hadamard_Bool
// hadamard.cpp:340-439 with SAFE_HASH
static void hadamard_bool(State& st, size_t out_id, const sq_cond* cond) {
    if (st.empty()) return;
    std::map<System, size_t, LessExceptKey> buckets(LessExceptKey{out_id});
    size_t current_size = st.size();
    auto op_pair = [&](size_t zero, size_t one) {
        complex_t a = st[zero].amplitude, b = st[one].amplitude;
        st[zero].amplitude = cscale(a, kSqrt2Inv) + cscale(b, kSqrt2Inv);
        st[one].amplitude = cscale(a, kSqrt2Inv) - cscale(b, kSqrt2Inv);
    };
    for (size_t i = 0; i < current_size; ++i) {
        if (!condition_satisfied(st[i], cond)) continue;
        auto iter = buckets.find(st[i]);
        if (iter == buckets.end()) { buckets.insert({st[i], i}); continue; }
        if (as_u64(st[iter->second].get(out_id), 1)) op_pair(i, iter->second);
        else op_pair(iter->second, i);
        buckets.erase(iter);
    }
    for (auto& kv : buckets) {
        size_t k = kv.second;
        if (as_u64(st[k].get(out_id), 1)) {  // operate_alone_one
            System c = st[k];
            st.push_back(c);
            st.back().get(out_id) = 0;
            st.back().amplitude = cscale(st.back().amplitude, kSqrt2Inv);
            st[k].amplitude = cscale(st[k].amplitude, -kSqrt2Inv);
        } else {  // operate_alone_zero
            System c = st[k];
            st.push_back(c);
            st.back().get(out_id) = 1;
            st[k].amplitude = cscale(st[k].amplitude, kSqrt2Inv);
            st.back().amplitude = cscale(st.back().amplitude, kSqrt2Inv);
        }
    }
    clear_zero(st, g_clearzero_eps);
}

// ---------------------------------------------------------------- Rot_Bool
// basic_gates.cpp:74-357 (the sort-based v1 path, use_hash = false)
static bool rot_is_diagonal(const complex_t* m) { return abs_sqr(m[1]) < kEpsilon && abs_sqr(m[2]) < kEpsilon; }
static bool rot_is_off_diagonal(const complex_t* m) { return abs_sqr(m[0]) < kEpsilon && abs_sqr(m[3]) < kEpsilon; }

static void rot_bool(State& st, size_t id, size_t digit, const complex_t* mat, const sq_cond* cond) {
    if (st.empty()) return;
    uint64_t mask = pow2(digit);
    // SortExceptBit (sort_state.cpp:52-78)
    auto pred = [id, digit](const System& l, const System& r) {
        uint64_t m = ~pow2(digit);
        for (size_t i = 0; i < g_regs.size(); ++i) {
            if (!status_of(i) || i == id) continue;
            if (l.get(i) < r.get(i)) return true;
            if (l.get(i) > r.get(i)) return false;
        }
        return (l.get(id) & m) < (r.get(id) & m);
    };
    std::sort(st.begin(), st.end(), pred);
    // compare_equal_rot (sort_state.cpp:212-232) with mask ~bit
    auto eq = [id, mask](const System& a, const System& b) {
        for (size_t i = g_regs.size(); i-- > 0;) {
            if (!status_of(i)) continue;
            if (i == id) {
                if ((a.get(id) & ~mask) != (b.get(id) & ~mask)) return false;
                continue;
            }
            if (a.get(i) != b.get(i)) return false;
        }
        return true;
    };
    auto operate = [&](size_t l, size_t r) {
        size_t n = r - l;
        if (n == 0) return;
        if (rot_is_diagonal(mat)) {
            for (size_t i = l; i < r; ++i) {
                if (!condition_satisfied(st[i], cond)) return;
                if (st[i].get(id) & mask) st[i].amplitude = cmul(st[i].amplitude, mat[3]);
                else st[i].amplitude = cmul(st[i].amplitude, mat[0]);
            }
        } else if (rot_is_off_diagonal(mat)) {
            for (size_t i = l; i < r; ++i) {
                if (!condition_satisfied(st[i], cond)) return;
                uint64_t& v = st[i].get(id);
                if (v & mask) { st[i].amplitude = cmul(st[i].amplitude, mat[1]); v ^= mask; }
                else { st[i].amplitude = cmul(st[i].amplitude, mat[2]); v ^= mask; }
            }
        } else if (n == 1) {
            if (!condition_satisfied(st[l], cond)) return;
            size_t new_pos = st.size();
            System c = st[l];
            st.push_back(c);
            bool v = st[l].get(id) & mask;
            st[new_pos].get(id) ^= mask;
            if (!v) {
                st[l].amplitude = cmul(st[l].amplitude, mat[0]);
                st[new_pos].amplitude = cmul(st[new_pos].amplitude, mat[2]);
            } else {
                st[new_pos].amplitude = cmul(st[new_pos].amplitude, mat[1]);
                st[l].amplitude = cmul(st[l].amplitude, mat[3]);
            }
        } else {
            if (!condition_satisfied(st[l], cond)) return;
            bool is_zero = get_as(st[l], id) & pow2(digit);
            complex_t a = st[l].amplitude, b = st[l + 1].amplitude;
            if (!is_zero) {
                st[l].amplitude = cmul(a, mat[0]) + cmul(b, mat[1]);
                st[l + 1].amplitude = cmul(a, mat[2]) + cmul(b, mat[3]);
            } else {
                st[l + 1].amplitude = cmul(b, mat[0]) + cmul(a, mat[1]);
                st[l].amplitude = cmul(b, mat[2]) + cmul(a, mat[3]);
            }
        }
    };
    size_t current_size = st.size();
    size_t l = 0, r = 1;
    while (true) {
        if (r == current_size) { operate(l, r); break; }
        if (!eq(st[l], st[r])) { operate(l, r); l = r; r = l + 1; }
        else r++;
    }
    clear_zero(st, g_clearzero_eps);
}

// ---------------------------------------------------------------- CondRot_Rational_Bool
// condrot.cpp:12-152 with SAFE_HASH
static void condrot(State& st, size_t reg_in, size_t reg_out, bool dag) {
    if (st.empty()) return;
    std::map<System, size_t, LessExceptKey> buckets(LessExceptKey{reg_out});
    double sgn = dag ? -2 * kPi : 2 * kPi;
    auto mapping = [](System& s0, System& s1, double c, double s) {
        complex_t a0 = s0.amplitude, a1 = s1.amplitude;
        s0.amplitude = cscale(a0, c) - cscale(a1, s);
        s1.amplitude = cscale(a0, s) + cscale(a1, c);
    };
    size_t current_size = st.size();
    for (size_t i = 0; i < current_size; ++i) {
        auto iter = buckets.find(st[i]);
        if (iter == buckets.end()) { buckets.insert({st[i], i}); continue; }
        size_t first = iter->second, second = i;
        bool first_one = as_u64(st[first].get(reg_out), size_of(reg_out)) != 0;
        size_t zero = first_one ? second : first;
        size_t one = first_one ? first : second;
        double rot = as_double(st[zero].get(reg_in), size_of(reg_in)) * sgn;
        mapping(st[zero], st[one], std::cos(rot), std::sin(rot));
        buckets.erase(iter);
    }
    for (auto& kv : buckets) {
        size_t original = kv.second;
        System c = st[original];
        st.push_back(c);
        st.back().get(reg_out) ^= 1;
        st.back().amplitude = 0;
        bool original_is_one = as_u64(st[original].get(reg_out), size_of(reg_out)) != 0;
        size_t zero = original_is_one ? st.size() - 1 : original;
        size_t one = original_is_one ? original : st.size() - 1;
        double rot = as_double(st[zero].get(reg_in), size_of(reg_in)) * sgn;
        mapping(st[zero], st[one], std::cos(rot), std::sin(rot));
    }
    clear_zero(st, g_clearzero_eps);
}

// ---------------------------------------------------------------- CondRot_General_Bool_Fast
// condrot.h:149-300 with SAFE_HASH; the callable is a table of 2x2 matrices
static void condrot_general(State& st, size_t in_id, size_t out_id, const complex_t* table) {
    if (st.empty()) return;
    std::map<System, size_t, LessExceptKey> buckets(LessExceptKey{out_id});
    auto mat_of = [&](size_t k) { return table + 4 * as_u64(st[k].get(in_id), size_of(in_id)); };
    auto op_pair = [&](size_t zero, size_t one) {
        const complex_t* m = mat_of(zero);
        complex_t a = st[zero].amplitude, b = st[one].amplitude;
        st[zero].amplitude = cmul(a, m[0]) + cmul(b, m[1]);
        st[one].amplitude = cmul(a, m[2]) + cmul(b, m[3]);
    };
    size_t current_size = st.size();
    for (size_t i = 0; i < current_size; ++i) {
        auto iter = buckets.find(st[i]);
        if (iter == buckets.end()) { buckets.insert({st[i], i}); continue; }
        if (as_u64(st[iter->second].get(out_id), 1)) op_pair(i, iter->second);
        else op_pair(iter->second, i);
        buckets.erase(iter);
    }
    for (auto& kv : buckets) {
        size_t k = kv.second;
        const complex_t* m = mat_of(k);
        System c = st[k];
        if (as_u64(st[k].get(out_id), 1)) {  // operate_alone_one
            st.push_back(c);
            st.back().get(out_id) = 0;
            st.back().amplitude = cmul(st.back().amplitude, m[1]);
            st[k].amplitude = cmul(st[k].amplitude, m[3]);
        } else {  // operate_alone_zero
            st.push_back(c);
            st.back().get(out_id) = 1;
            st[k].amplitude = cmul(st[k].amplitude, m[0]);
            st.back().amplitude = cmul(st.back().amplitude, m[2]);
        }
    }
    clear_zero(st, g_clearzero_eps);
}

// ---------------------------------------------------------------- Rot_GeneralUnitary
// rot.cpp:353-477 with SAFE_HASH
static void rot_general_unitary(State& st, size_t id, const complex_t* mat, bool dagger, const sq_cond* cond) {
    if (st.empty()) return;
    size_t full_size = (size_t)pow2(size_of(id));
    auto bucket_op = [&](const std::vector<size_t>& positions) {
        std::vector<complex_t> amps(positions.size());
        for (size_t i = 0; i < positions.size(); ++i) amps[i] = st[positions[i]].amplitude;
        std::vector<complex_t> new_amps(positions.size(), 0);
        for (size_t i = 0; i < full_size; ++i)
            for (size_t j = 0; j < full_size; ++j) {
                complex_t m = dagger ? std::conj(mat[j * full_size + i]) : mat[i * full_size + j];
                new_amps[i] += cmul(m, amps[j]);
            }
        for (size_t i = 0; i < positions.size(); ++i) st[positions[i]].amplitude = new_amps[i];
    };
    std::map<System, std::pair<size_t, std::vector<size_t>>, LessExceptKey> buckets(LessExceptKey{id});
    size_t current_size = st.size();
    for (size_t i = 0; i < current_size; ++i) {
        if (!condition_satisfied(st[i], cond)) continue;
        uint64_t val = get_as(st[i], id);
        auto res = buckets.insert({st[i], {0, std::vector<size_t>(full_size, (size_t)-1)}});
        auto iter = res.first;
        iter->second.second[val] = i;
        iter->second.first += 1;
        if (iter->second.first == full_size) {
            bucket_op(iter->second.second);
            buckets.erase(iter);
        }
    }
    for (auto& kv : buckets) {
        auto& all_pos = kv.second.second;
        for (size_t i = 0; i < all_pos.size(); ++i)
            if (all_pos[i] == (size_t)-1) {
                st.push_back(kv.first);
                st.back().get(id) = i;
                st.back().amplitude = 0;
                all_pos[i] = st.size() - 1;
            }
        bucket_op(all_pos);
    }
    clear_zero(st, g_clearzero_eps);
}

// ---------------------------------------------------------------- Hadamard_Partial
// One position: the pair arithmetic of the reference's active path,
// Hadamard_Partial::operator() with use_hash (hadamard.cpp:619-711): entries
// equal except the chosen bit combined as a*sqrt2inv +- b*sqrt2inv
// (operate_pair), lone entries given their partner (operate_alone_zero /
// _one). The reference's buckets never actually pair two entries (their
// order, StateLessExceptQubits, ends on the whole register,
// quantum_interfere_basic.cpp:151-177), so it leaves partners as duplicate
// keys; here they are paired, which is the transform, and equals the
// reference wherever no two entries are partners. That path also never tests
// the operator's conditions; this restatement leaves the entries that fail
// them untouched (every other controllable split operator of the reference
// does so), which is the same result wherever no condition is set.
static void hadamard_partial1(State& st, size_t id, size_t pos, const sq_cond* cond) {
    if (st.empty()) return;
    uint64_t bit = pow2(pos);
    struct Less {
        size_t id;
        uint64_t bit;
        bool operator()(const System& a, const System& b) const {
            for (size_t i = 0; i < g_regs.size(); ++i) {
                if (!status_of(i)) continue;
                uint64_t x = a.get(i), y = b.get(i);
                if (i == id) { x &= ~bit; y &= ~bit; }
                if (x < y) return true;
                if (x > y) return false;
            }
            return false;
        }
    };
    std::map<System, size_t, Less> buckets(Less{id, bit});
    auto op_pair = [&](size_t zero, size_t one) {
        complex_t a = st[zero].amplitude, b = st[one].amplitude;
        st[zero].amplitude = cscale(a, kSqrt2Inv) + cscale(b, kSqrt2Inv);
        st[one].amplitude = cscale(a, kSqrt2Inv) - cscale(b, kSqrt2Inv);
    };
    size_t current_size = st.size();
    for (size_t i = 0; i < current_size; ++i) {
        if (!condition_satisfied(st[i], cond)) continue;
        auto iter = buckets.find(st[i]);
        if (iter == buckets.end()) { buckets.insert({st[i], i}); continue; }
        if (st[iter->second].get(id) & bit) op_pair(i, iter->second);
        else op_pair(iter->second, i);
        buckets.erase(iter);
    }
    for (auto& kv : buckets) {
        size_t k = kv.second;
        System c = st[k];
        if (st[k].get(id) & bit) {  // operate_alone_one
            st.push_back(c);
            st.back().get(id) &= ~bit;
            st.back().amplitude = cscale(st.back().amplitude, kSqrt2Inv);
            st[k].amplitude = cscale(st[k].amplitude, -kSqrt2Inv);
        } else {  // operate_alone_zero
            st.push_back(c);
            st.back().get(id) |= bit;
            st[k].amplitude = cscale(st[k].amplitude, kSqrt2Inv);
            st.back().amplitude = cscale(st.back().amplitude, kSqrt2Inv);
        }
    }
    clear_zero(st, g_clearzero_eps);
}

// Several positions: H on each bit of the set, Hadamard_Partial::operate
// (hadamard.cpp:468-570) over the groups of SortExceptKeyHadamard
// (sort_state.cpp:133-170; equal on every other register and on the
// register's bits outside the set, members in ascending value). Member
// index i of a group is the set's bits of its value gathered in ascending
// position order (from_map_position, hadamard.cpp:457-466); the group's
// fan-out writes index i back at those positions (map_position, :443-452).
// The three cases (one member, a full group, the rest) and their butterfly
// order are the reference's. The one-member sign is (-1)^popcount(i & v):
// the reference's expression there, bitcount(i & v & 1), reads only bit 0
// of i & v, which is the same for one position and not the Hadamard
// transform for more (that code path is compiled but not the one the
// operator runs; the reference's QASM front end merges runs of single-qubit
// h gates into one Hadamard_Partial, which needs the transform).
static uint64_t hp_map_position(uint64_t i, const std::vector<size_t>& pos) {
    uint64_t v = 0;
    for (size_t k = 0; k < pos.size(); ++k) v |= ((i >> k) & 1ull) << pos[k];
    return v;
}
static uint64_t hp_from_map_position(uint64_t v, const std::vector<size_t>& pos) {
    uint64_t i = 0;
    for (size_t k = 0; k < pos.size(); ++k) i |= ((v >> pos[k]) & 1ull) << k;
    return i;
}
static void hadamard_partial_operate(size_t l, size_t r, State& st, size_t id, const std::vector<size_t>& pos,
                                     uint64_t mask, const sq_cond* cond) {
    size_t n = r - l;
    size_t full_size = (size_t)pow2(pos.size());
    size_t original_size = st.size();
    double extra_amplitude = 1.0 / std::sqrt((double)full_size);
    if (n == 0) return;
    if (!condition_satisfied(st[l], cond)) return;
    if (n == 1) {
        uint64_t v = hp_from_map_position(st[l].get(id), pos);
        st[l].amplitude = cscale(st[l].amplitude, extra_amplitude);
        System base = st[l];
        st.insert(st.end(), full_size, base);
        for (size_t i = 0; i < full_size; ++i) {
            size_t p = original_size + i;
            st[p].get(id) = (st[p].get(id) & mask) + hp_map_position(i, pos);
            if (bitcount(i & v) & 1) st[p].amplitude = complex_t(st[p].amplitude.real() * -1, st[p].amplitude.imag() * -1);
        }
        st[l].amplitude = 0;
    } else if (n == full_size) {
        for (size_t qn = 0; qn < pos.size(); ++qn)
            for (size_t i = 0; i < full_size; ++i)
                if ((i >> qn) & 1) {
                    complex_t a0 = st[i + l - pow2(qn)].amplitude, a1 = st[i + l].amplitude;
                    st[i + l - pow2(qn)].amplitude = cscale(a0 + a1, kSqrt2Inv);
                    st[i + l].amplitude = cscale(a0 - a1, kSqrt2Inv);
                }
    } else {
        System base = st[l];
        st.insert(st.end(), full_size, base);
        uint64_t value_mask = st[l].get(id) & mask;
        for (size_t i = 0; i < full_size; ++i) {
            st[i + original_size].amplitude = 0;
            st[i + original_size].get(id) = value_mask + hp_map_position(i, pos);
        }
        for (size_t i = l; i < r; ++i) {
            st[hp_from_map_position(st[i].get(id), pos) + original_size].amplitude = st[i].amplitude;
            st[i].amplitude = 0;
        }
        for (size_t qn = 0; qn < pos.size(); ++qn)
            for (size_t i = 0; i < full_size; ++i)
                if ((i >> qn) & 1) {
                    complex_t a0 = st[i + original_size - pow2(qn)].amplitude, a1 = st[i + original_size].amplitude;
                    st[i + original_size - pow2(qn)].amplitude = cscale(a0 + a1, kSqrt2Inv);
                    st[i + original_size].amplitude = cscale(a0 - a1, kSqrt2Inv);
                }
    }
}
static void hadamard_partial_multi(State& st, size_t id, std::vector<size_t> pos, const sq_cond* cond) {
    if (st.empty()) return;
    uint64_t setbits = 0;
    for (size_t p : pos) setbits |= pow2(p);
    const uint64_t mask = ~setbits;  // make_mask: every bit outside the set
    auto pred = [&](const System& a, const System& b) {
        for (size_t i = 0; i < g_regs.size(); ++i) {
            if (!status_of(i)) continue;
            uint64_t x = a.get(i), y = b.get(i);
            if (i == id) { x &= mask; y &= mask; }
            if (x < y) return true;
            if (x > y) return false;
        }
        return a.get(id) < b.get(id);
    };
    auto same = [&](const System& a, const System& b) {  // compare_equal_hadamard
        for (size_t i = 0; i < g_regs.size(); ++i) {
            if (!status_of(i)) continue;
            uint64_t x = a.get(i), y = b.get(i);
            if (i == id) { x &= mask; y &= mask; }
            if (x != y) return false;
        }
        return true;
    };
    std::sort(st.begin(), st.end(), pred);
    size_t current_size = st.size();
    size_t l = 0, r = 1;
    while (true) {
        if (r == current_size) { hadamard_partial_operate(l, r, st, id, pos, mask, cond); break; }
        if (!same(st[l], st[r])) {
            hadamard_partial_operate(l, r, st, id, pos, mask, cond);
            l = r;
            r = l + 1;
        } else {
            r++;
        }
    }
    clear_zero(st, g_clearzero_eps);
}

// ---------------------------------------------------------------- Normalize / add_systems
static double normalize(State& st) {  // dark_magic.cpp:11-32
    double sum_prob = 0.0;
    for (const auto& s : st) sum_prob += abs_sqr(s.amplitude);
    double k = 1.0 / std::sqrt(sum_prob);
    if (std::isnan(k)) throw std::runtime_error("bad result");
    for (auto& s : st) s.amplitude = cscale(s.amplitude, k);
    return sum_prob;
}

static bool system_less(const System& a, const System& b) {  // basic_components.cpp:463-476
    for (size_t i = 0; i < g_regs.size(); ++i) {
        if (!status_of(i)) continue;
        if (a.get(i) < b.get(i)) return true;
        if (b.get(i) < a.get(i)) return false;
    }
    return false;
}
static bool system_equal(const System& a, const System& b) {
    for (size_t i = 0; i < g_regs.size(); ++i) {
        if (!status_of(i)) continue;
        if (a.get(i) != b.get(i)) return false;
    }
    return true;
}

static void add_systems(State& cur, const State& add, double coef) {  // system_operations.h:157-175
    if (add.empty()) return;
    size_t original_size = cur.size();
    cur.insert(cur.end(), add.begin(), add.end());
    if (std::abs(coef - 1.0) > kEpsilon)
        for (size_t i = original_size; i < cur.size(); ++i) cur[i].amplitude = cscale(cur[i].amplitude, coef);
    if (original_size == 0) return;
    // sort_merge_unique_erase: stable sort keeps the current state's entry
    // ahead of the added one, so runs sum in (current, added) order.
    std::stable_sort(cur.begin(), cur.end(), system_less);
    State out;
    out.reserve(cur.size());
    for (size_t i = 0; i < cur.size();) {
        size_t j = i + 1;
        System acc = cur[i];
        while (j < cur.size() && system_equal(cur[i], cur[j])) { acc.amplitude += cur[j].amplitude; ++j; }
        if (!(abs_sqr(acc.amplitude) < kEpsilon)) out.push_back(acc);
        i = j;
    }
    cur.swap(out);
}

// ---------------------------------------------------------------- registers
static size_t add_register(uint32_t type, size_t size) {  // basic_components.cpp:330-364
    if (!g_reusable.empty()) {
        size_t id = g_reusable.back();
        g_reusable.pop_back();
        g_regs[id] = {type, size, true};
        return id;
    }
    g_regs.push_back({type, size, true});
    return g_regs.size() - 1;
}
static void remove_register(size_t id) {  // basic_components.cpp:378-389
    if (id >= g_regs.size() || !g_regs[id].active) throw std::invalid_argument("register not active");
    g_regs[id].active = false;
    g_reusable.push_back(id);
}

}  // namespace sqo

// ====================================================================== C API
using namespace sqo;

#define SQO_TRY(...)                                    \
    try {                                               \
        __VA_ARGS__;                                    \
        return 0;                                       \
    } catch (const std::exception& e) {                 \
        g_err = e.what();                               \
        return 1;                                       \
    }

extern "C" {

const char* sqo_last_error(void) { return g_err.c_str(); }

int sqo_clear(void) {
    g_regs.clear();
    g_reusable.clear();
    g_clearzero_eps = kEpsilon;
    return 0;
}
int sqo_set_clearzero_eps(double eps) { g_clearzero_eps = eps; return 0; }
int sqo_add_register(uint32_t type, uint32_t width, uint32_t* id) {
    SQO_TRY(if (width > 64) throw std::invalid_argument("width > 64"); *id = (uint32_t)add_register(type, width))
}
int sqo_remove_register(uint32_t id) { SQO_TRY(remove_register(id)) }
int sqo_register_count(uint32_t* n) { *n = (uint32_t)g_regs.size(); return 0; }
int sqo_register_info(uint32_t id, uint32_t* type, uint32_t* width, uint32_t* active) {
    SQO_TRY(const RegInfo& r = g_regs.at(id); *type = r.type; *width = (uint32_t)r.size; *active = r.active)
}

void* sqo_state_new(void) { return new State(1); }
void sqo_state_free(void* h) { delete static_cast<State*>(h); }
uint64_t sqo_state_size(void* h) { return static_cast<State*>(h)->size(); }
int sqo_state_copy(void* dst, const void* src) {
    *static_cast<State*>(dst) = *static_cast<const State*>(src);
    return 0;
}
int sqo_state_set(void* h, uint64_t n, const uint64_t* regs, uint32_t nregs, const double* amps) {
    SQO_TRY({
        State& st = *static_cast<State*>(h);
        st.assign(n, System());
        for (uint64_t i = 0; i < n; ++i) {
            st[i].amplitude = complex_t(amps[2 * i], amps[2 * i + 1]);
            for (uint32_t r = 0; r < nregs; ++r) st[i].get(r) = regs[i * nregs + r];
        }
    })
}
int sqo_state_get(void* h, uint64_t* regs, uint32_t nregs, double* amps) {
    SQO_TRY({
        State& st = *static_cast<State*>(h);
        for (size_t i = 0; i < st.size(); ++i) {
            amps[2 * i] = st[i].amplitude.real();
            amps[2 * i + 1] = st[i].amplitude.imag();
            for (uint32_t r = 0; r < nregs; ++r) regs[(size_t)i * nregs + r] = r < g_regs.size() ? st[i].get(r) : 0;
        }
    })
}

void* sqo_qram_new(uint32_t address_size, uint32_t data_size, const uint64_t* memory, uint64_t n) {
    Qram* q = new Qram{address_size, data_size, std::vector<uint64_t>(memory, memory + n)};
    return q;
}
void sqo_qram_free(void* q) { delete static_cast<Qram*>(q); }

int sqo_apply(void* h, const sq_instr* prog, uint32_t n) {
    SQO_TRY(for (uint32_t i = 0; i < n; ++i) apply_instr(*static_cast<State*>(h), prog[i]))
}
int sqo_hadamard_int(void* h, uint32_t reg, uint32_t n_digits, const sq_cond* cond) {
    SQO_TRY(hadamard_int(*static_cast<State*>(h), reg, n_digits, cond))
}
int sqo_hadamard_int_full(void* h, uint32_t reg, const sq_cond* cond) {
    SQO_TRY(hadamard_int_full(*static_cast<State*>(h), reg, cond))
}
int sqo_hadamard_bool(void* h, uint32_t reg, const sq_cond* cond) {
    SQO_TRY(hadamard_bool(*static_cast<State*>(h), reg, cond))
}
int sqo_rot_bool(void* h, uint32_t reg, uint32_t digit, const double* m8, const sq_cond* cond, int dag) {
    SQO_TRY({
        complex_t m[4] = {{m8[0], m8[1]}, {m8[2], m8[3]}, {m8[4], m8[5]}, {m8[6], m8[7]}};
        if (dag) {  // u22_t::dagger: conjugate transpose
            complex_t d[4] = {std::conj(m[0]), std::conj(m[2]), std::conj(m[1]), std::conj(m[3])};
            std::copy(d, d + 4, m);
        }
        rot_bool(*static_cast<State*>(h), reg, digit, m, cond);
    })
}
// With conditions: SPLIT_BY_CONDITIONS / MERGE_BY_CONDITIONS
// (system_operations.h:109-129) around the operator, as the reference's
// composite operators apply it: the entries failing the conditions are set
// aside, the operator (and its ClearZero) runs on the rest, they come back.
int sqo_condrot(void* h, uint32_t reg_in, uint32_t reg_out, int dag, const sq_cond* cond) {
    SQO_TRY({
        State& st = *static_cast<State*>(h);
        if (!cond || cond->count == 0) {
            condrot(st, reg_in, reg_out, dag != 0);
        } else {
            State pass, rest;
            for (auto& e : st) (condition_satisfied(e, cond) ? pass : rest).push_back(e);
            condrot(pass, reg_in, reg_out, dag != 0);
            pass.insert(pass.end(), rest.begin(), rest.end());
            st.swap(pass);
        }
    })
}
// with conditions: the entries that satisfy them are rotated (and pruned) as
// a state of their own, the others kept as they are (the partition of the
// reference's SPLIT_BY_CONDITIONS / MERGE_BY_CONDITIONS, system_operations.h:109-129)
int sqo_condrot_general(void* h, uint32_t reg_in, uint32_t reg_out, const double* table, uint64_t n_values,
                        const sq_cond* cond) {
    SQO_TRY({
        if (n_values != pow2(size_of(reg_in))) throw std::invalid_argument("table size");
        std::vector<complex_t> t(4 * n_values);
        for (uint64_t i = 0; i < 4 * n_values; ++i) t[i] = complex_t(table[2 * i], table[2 * i + 1]);
        State& st = *static_cast<State*>(h);
        if (!cond || cond->count == 0) {
            condrot_general(st, reg_in, reg_out, t.data());
        } else {
            State pass, rest;
            for (auto& e : st) (condition_satisfied(e, cond) ? pass : rest).push_back(e);
            condrot_general(pass, reg_in, reg_out, t.data());
            pass.insert(pass.end(), rest.begin(), rest.end());
            st.swap(pass);
        }
    })
}
int sqo_rot_general_unitary(void* h, uint32_t reg, const double* mat, uint64_t dim, const sq_cond* cond, int dag) {
    SQO_TRY({
        if (dim != pow2(size_of(reg))) throw std::invalid_argument("matrix size");
        std::vector<complex_t> m(dim * dim);
        for (uint64_t i = 0; i < dim * dim; ++i) m[i] = complex_t(mat[2 * i], mat[2 * i + 1]);
        rot_general_unitary(*static_cast<State*>(h), reg, m.data(), dag != 0, cond);
    })
}
int sqo_hadamard_partial(void* h, uint32_t reg, const uint32_t* positions, uint32_t n, const sq_cond* cond) {
    SQO_TRY({
        std::set<size_t> ps(positions, positions + n);  // the reference takes a std::set
        for (size_t p : ps)
            if (p >= size_of(reg)) throw std::invalid_argument("position >= register size");
        if (ps.empty()) return 0;
        if (ps.size() == 1) hadamard_partial1(*static_cast<State*>(h), reg, *ps.begin(), cond);
        else hadamard_partial_multi(*static_cast<State*>(h), reg, std::vector<size_t>(ps.begin(), ps.end()), cond);
    })
}
int sqo_clear_zero(void* h, double eps) { SQO_TRY(clear_zero(*static_cast<State*>(h), eps)) }
int sqo_partial_trace_select(void* h, const uint32_t* regs, const uint64_t* values, uint32_t n, int range,
                             uint64_t lo, uint64_t hi, double* result) {
    SQO_TRY({
        std::vector<uint32_t> r(regs, regs + n);
        std::vector<uint64_t> v;
        if (values) v.assign(values, values + n);
        *result = partial_trace_select(*static_cast<State*>(h), r, v, range != 0, lo, hi);
    })
}
int sqo_get_output(void* h, const uint32_t* zero, uint32_t n_zero, const uint32_t* idx, uint32_t n_idx,
                   double* out, uint64_t out_len, double* prob) {
    SQO_TRY({
        std::vector<complex_t> v;
        *prob = get_output(*static_cast<State*>(h), std::vector<uint32_t>(zero, zero + n_zero),
                           std::vector<uint32_t>(idx, idx + n_idx), v);
        if (v.size() != out_len) throw std::invalid_argument("out_len");
        for (size_t i = 0; i < v.size(); ++i) {
            out[2 * i] = v[i].real();
            out[2 * i + 1] = v[i].imag();
        }
    })
}
int sqo_qw_rotate_angle(void* h, uint32_t data, uint32_t out, uint32_t data_size, int positive_only,
                        const sq_cond* cond) {
    SQO_TRY(qw_rotate_angle(*static_cast<State*>(h), data, out, data_size, positive_only != 0, cond))
}
int sqo_normalize(void* h, double* norm_sq) {
    SQO_TRY({ double s = normalize(*static_cast<State*>(h)); if (norm_sq) *norm_sq = s; })
}
int sqo_add_systems(void* dst, const void* src, double coef) {
    SQO_TRY(add_systems(*static_cast<State*>(dst), *static_cast<const State*>(src), coef))
}
int sqo_add_register_sync(void* h, uint32_t type, uint32_t width, uint32_t* id) {
    SQO_TRY({
        size_t r = add_register(type, width);
        for (auto& s : *static_cast<State*>(h)) s.get(r) = 0;
        *id = (uint32_t)r;
    })
}
int sqo_remove_register_sync(void* h, uint32_t id) {
    SQO_TRY({
        for (auto& s : *static_cast<State*>(h)) s.get(id) = 0;
        remove_register(id);
    })
}
// SplitRegister::operator() (system_operations.cpp:124-158)
int sqo_split_register(void* h, uint32_t first, uint32_t second_size, uint32_t* second_out) {
    SQO_TRY({
        State& st = *static_cast<State*>(h);
        size_t original = size_of(first);
        if (original < second_size) throw std::invalid_argument("split larger than register");
        size_t second = add_register(g_regs[first].type, second_size);
        for (auto& s : st) s.get(second) = 0;
        g_regs[first].size = original - second_size;
        for (auto& s : st) {
            uint64_t& v = s.get(first);
            uint64_t m = second_size == 64 ? ~uint64_t{0} : pow2(second_size) - 1;
            s.get(second) = v & m;
            v = second_size == 64 ? 0 : v >> second_size;
        }
        *second_out = (uint32_t)second;
    })
}
// CombineRegister::operator() (system_operations.cpp:170-203)
int sqo_combine_register(void* h, uint32_t first, uint32_t second) {
    SQO_TRY({
        State& st = *static_cast<State*>(h);
        size_t fs = size_of(first), ss = size_of(second);
        if (fs + ss > 64) throw std::invalid_argument("combined width > 64");
        g_regs[first].size = fs + ss;
        for (auto& s : st) {
            uint64_t& v = s.get(first);
            uint64_t fm = fs == 64 ? ~uint64_t{0} : pow2(fs) - 1;
            uint64_t sm = ss == 64 ? ~uint64_t{0} : pow2(ss) - 1;
            uint64_t fv = v & fm, sv = s.get(second) & sm;
            v = ss == 64 ? sv : (fv << ss) | sv;
        }
        remove_register(second);
    })
}

}  // extern "C"
