// reference_driver.cpp — TEST INFRASTRUCTURE ONLY (oracle/). C entry points
// over the reference's own CPU operator classes (SparQ/src/*.cpp, compiled
// unmodified from where they lie, against the stand-in header in refshim/),
// so that a test can run one operation on the oracle (sparq_oracle.cpp) and on
// the reference and compare the two states bit for bit. Built by
// build_reference.py into oracle/_ref/libsparq_ref.so; never linked into, or
// loaded by, the engine.
//
// Conventions: register ids are the reference's System ids; a state is a
// std::vector<System>; an elementwise instruction uses the engine's sq_instr
// layout (include/sparq_gb300.h), the same one the oracle's sqo_apply reads,
// and is turned into the reference operator that opcode restates.
#include <cstring>
#include <memory>
#include <set>
#include <string>
#include <vector>

#include "sparse_state_simulator.h"
#include "sparq_gb300.h"

using namespace qram_simulator;

namespace {

std::string g_err;
uint64_t g_names = 0;  // reference registers need unique names

using State = std::vector<System>;

template <typename Op>
void with_cond_impl(Op& op, const sq_cond* c) {
    for (uint32_t i = 0; i < c->count; ++i) {
        const sq_condition& q = c->c[i];
        switch (q.kind) {
            case SQ_COND_NONZERO: op.condition_variable_nonzeros.push_back(q.reg); break;
            case SQ_COND_ALL_ONES: op.condition_variable_all_ones.push_back(q.reg); break;
            case SQ_COND_BIT: op.condition_variable_by_bit.emplace_back(q.reg, (size_t)q.param); break;
            case SQ_COND_VALUE: op.condition_variable_by_value.emplace_back(q.reg, (size_t)q.param); break;
            default: throw std::invalid_argument("condition kind");
        }
    }
}

template <typename Op>
Op& with_cond(Op& op, const sq_cond* c) {
    if (!c || c->count == 0) return op;
    if constexpr (!requires { op.condition_variable_nonzeros; }) {
        throw std::invalid_argument("the reference operator takes no conditions");
    } else {
        with_cond_impl(op, c);
    }
    return op;
}

template <typename Op>
void run(Op op, State& st, const sq_cond* c, bool dag) {
    with_cond(op, c);
    if (dag) op.dag(st);
    else op(st);
}

StateStorageType to_type(uint32_t t) {
    switch (t) {
        case SQ_GENERAL: return General;
        case SQ_UNSIGNED: return UnsignedInteger;
        case SQ_SIGNED: return SignedInteger;
        case SQ_BOOLEAN: return Boolean;
        case SQ_RATIONAL: return Rational;
    }
    throw std::invalid_argument("register type");
}

// the register ids of a bitmask (the reflections' imm0)
std::vector<size_t> mask_ids(uint64_t m) {
    std::vector<size_t> ids;
    for (size_t id = 0; id < 64; ++id)
        if ((m >> id) & 1) ids.push_back(id);
    return ids;
}

void apply_one(State& st, const sq_instr& in) {
    const uint32_t* r = in.reg;
    const uint64_t* im = in.imm;
    const sq_cond* c = &in.cond;
    const bool d = in.dag != 0;
    switch (in.op) {
        case SQ_OP_NOP: return;
        case SQ_OP_FLIP_BOOLS: return run(FlipBools(r[0]), st, c, false);
        case SQ_OP_SWAP_BOOL_BOOL: return run(Swap_Bool_Bool(r[0], im[0], r[1], im[1]), st, c, false);
        case SQ_OP_SHIFT_LEFT: return run(ShiftLeft_InPlace(r[0], im[0]), st, c, d);
        case SQ_OP_SHIFT_RIGHT: return run(ShiftRight_InPlace(r[0], im[0]), st, c, d);
        case SQ_OP_MULT_UINT_CONST: return run(Mult_UInt_ConstUInt(r[0], im[0], r[2]), st, c, false);
        case SQ_OP_ADD_MULT_UINT_CONST: return run(Add_Mult_UInt_ConstUInt_InPlace(r[0], im[0], r[2]), st, c, d);
        case SQ_OP_ADD_UINT_UINT: return run(Add_UInt_UInt(r[0], r[1], r[2]), st, c, false);
        case SQ_OP_ADD_UINT_UINT_INPLACE: return run(Add_UInt_UInt_InPlace(r[0], r[1]), st, c, d);
        case SQ_OP_ADD_UINT_CONST: return run(Add_UInt_ConstUInt(r[0], im[0], r[2]), st, c, false);
        case SQ_OP_ADD_CONST_INPLACE: return run(Add_ConstUInt_InPlace(r[0], im[0]), st, c, d);
        case SQ_OP_SUB_UINT_UINT: return run(Sub_UInt_UInt(r[0], r[1], r[2]), st, c, false);
        case SQ_OP_NEG_UINT: return run(Neg_UInt(r[0], r[1]), st, c, false);
        case SQ_OP_ABS_SINT: return run(Abs_SInt(r[0], r[1]), st, c, false);
        case SQ_OP_MUL_UINT_UINT: return run(Mul_UInt_UInt(r[0], r[1], r[2]), st, c, false);
        case SQ_OP_DIV_UINT_UINT: return run(Div_UInt_UInt(r[0], r[1], r[2]), st, c, false);
        case SQ_OP_SQRT_UINT: return run(Sqrt_UInt(r[0], r[1]), st, c, false);
        case SQ_OP_SELECT_BOOL: return run(Select_Bool_UInt_UInt(r[0], r[1], r[2], r[3]), st, c, false);
        case SQ_OP_AND_UINT_UINT: return run(And_UInt_UInt(r[0], r[1], r[2]), st, c, false);
        case SQ_OP_OR_UINT_UINT: return run(Or_UInt_UInt(r[0], r[1], r[2]), st, c, false);
        case SQ_OP_XOR_UINT_UINT: return run(Xor_UInt_UInt(r[0], r[1], r[2]), st, c, false);
        case SQ_OP_LESS_SINT_SINT: return run(Less_SInt_SInt(r[0], r[1], r[2]), st, c, false);
        case SQ_OP_CARRY_UINT_UINT: return run(Carry_UInt_UInt(r[0], r[1], r[2], r[3]), st, c, false);
        case SQ_OP_OVERFLOW_SINT_SINT: return run(Overflow_SInt_SInt(r[0], r[1], r[2], r[3]), st, c, false);
        case SQ_OP_MULOVERFLOW_UINT_UINT: return run(MulOverflow_UInt_UInt(r[0], r[1], r[2], r[3]), st, c, false);
        case SQ_OP_ISZERO_UINT: return run(IsZero_UInt(r[0], r[1]), st, c, false);
        case SQ_OP_NEGATIVE_SINT: return run(Negative_SInt(r[0], r[1]), st, c, false);
        case SQ_OP_ADD_ANYINT_INPLACE: return run(Add_AnyInt_AnyInt_InPlace(r[0], r[1]), st, c, d);
        case SQ_OP_ASSIGN: return run(Assign(r[0], r[1]), st, c, false);
        case SQ_OP_COMPARE_UINT_UINT: return run(Compare_UInt_UInt(r[0], r[1], r[2], r[3]), st, c, false);
        case SQ_OP_LESS_UINT_UINT: return run(Less_UInt_UInt(r[0], r[1], r[2]), st, c, false);
        case SQ_OP_SWAP_GENERAL: return run(Swap_General_General(r[0], r[1]), st, c, false);
        case SQ_OP_GETMID_UINT_UINT: return run(GetMid_UInt_UInt(r[0], r[1], r[2]), st, c, false);
        case SQ_OP_X_BOOL: return run(X_Bool(r[0], im[0]), st, c, false);
        case SQ_OP_Y_BOOL: return run(Y_Bool(r[0], im[0]), st, c, false);
        case SQ_OP_ANGLE_XOR:
            if (im[0] == 0) return run(Div_Sqrt_Arccos_UInt_UInt(r[0], r[1], r[2]), st, c, false);
            return run(GetRotateAngle_Int_Int(r[0], r[1], r[2]), st, c, false);
        case SQ_OP_REFLECTION_BOOL:
            return run(Reflection_Bool(mask_ids(im[0]), im[1] != 0), st, c, false);
        case SQ_OP_ZERO_COND_PHASE_FLIP:
            return run(ZeroConditionalPhaseFlip(mask_ids(im[0])), st, c, false);
        default: throw std::invalid_argument("opcode not driven through the reference: " + std::to_string(in.op));
    }
}

}  // namespace

#define REF_TRY(body)                 \
    try {                             \
        body;                         \
        return 0;                     \
    } catch (const std::exception& e) { \
        g_err = e.what();             \
        return 1;                     \
    } catch (...) {                   \
        g_err = "unknown error";      \
        return 1;                     \
    }

extern "C" {

const char* ref_last_error(void) { return g_err.c_str(); }

// ---------------------------------------------------------------- register table (System, basic_components.cpp)
int ref_clear(void) { REF_TRY(System::clear()) }
int ref_set_clearzero_eps(double eps) { REF_TRY(clearzero_default_eps = eps) }
int ref_add_register(uint32_t type, uint32_t width, uint32_t* id) {
    REF_TRY({
        *id = (uint32_t)System::add_register("r" + std::to_string(g_names++), to_type(type), width);
    })
}
int ref_register_count(uint32_t* n) { REF_TRY(*n = (uint32_t)System::name_register_map.size()) }

// ---------------------------------------------------------------- states
void* ref_state_new(void) { return new State(1); }
void ref_state_free(void* h) { delete static_cast<State*>(h); }
uint64_t ref_state_size(void* h) { return static_cast<State*>(h)->size(); }
int ref_state_set(void* h, uint64_t n, const uint64_t* regs, uint32_t nregs, const double* amps) {
    REF_TRY({
        State& st = *static_cast<State*>(h);
        st.assign(n, System());
        for (uint64_t i = 0; i < n; ++i) {
            for (uint32_t k = 0; k < nregs; ++k) st[i].get(k).value = regs[i * nregs + k];
            st[i].amplitude = complex_t(amps[2 * i], amps[2 * i + 1]);
        }
    })
}
int ref_state_get(void* h, uint64_t* regs, uint32_t nregs, double* amps) {
    REF_TRY({
        State& st = *static_cast<State*>(h);
        for (size_t i = 0; i < st.size(); ++i) {
            for (uint32_t k = 0; k < nregs; ++k) regs[i * nregs + k] = st[i].get(k).value;
            amps[2 * i] = st[i].amplitude.real();
            amps[2 * i + 1] = st[i].amplitude.imag();
        }
    })
}

// ---------------------------------------------------------------- operations
int ref_apply(void* h, const sq_instr* prog, uint32_t n) {
    REF_TRY({
        State& st = *static_cast<State*>(h);
        for (uint32_t i = 0; i < n; ++i) apply_one(st, prog[i]);
    })
}
int ref_qram_load(void* h, uint32_t address_size, uint32_t data_size, const uint64_t* mem, uint64_t nmem,
                  uint32_t reg_addr, uint32_t reg_data, const sq_cond* c) {
    REF_TRY({
        qram_qutrit::QRAMCircuit q(address_size, data_size, std::vector<uint64_t>(mem, mem + nmem));
        run(QRAMLoad(&q, reg_addr, reg_data), *static_cast<State*>(h), c, false);
    })
}
int ref_phase_bool(void* h, uint32_t reg, uint32_t digit, double lambda, int dag, const sq_cond* c) {
    REF_TRY(run(Phase_Bool(reg, digit, lambda), *static_cast<State*>(h), c, dag != 0))
}
int ref_global_phase(void* h, double re, double im, const sq_cond* c) {
    REF_TRY(run(GlobalPhase(complex_t(re, im)), *static_cast<State*>(h), c, false))
}
int ref_hadamard_int(void* h, uint32_t reg, uint32_t n, const sq_cond* c) {
    REF_TRY(run(Hadamard_Int(reg, n), *static_cast<State*>(h), c, false))
}
int ref_hadamard_int_full(void* h, uint32_t reg, const sq_cond* c) {
    REF_TRY(run(Hadamard_Int_Full(reg), *static_cast<State*>(h), c, false))
}
int ref_hadamard_bool(void* h, uint32_t reg, const sq_cond* c) {
    REF_TRY(run(Hadamard_Bool(reg), *static_cast<State*>(h), c, false))
}
int ref_hadamard_partial(void* h, uint32_t reg, const uint32_t* pos, uint32_t npos, const sq_cond* c) {
    REF_TRY({
        std::set<size_t> p(pos, pos + npos);
        run(Hadamard_Partial(reg, p), *static_cast<State*>(h), c, false);
    })
}
int ref_rot_bool(void* h, uint32_t reg, uint32_t digit, const double* m8, int dag, const sq_cond* c) {
    REF_TRY({
        u22_t m(complex_t(m8[0], m8[1]), complex_t(m8[2], m8[3]), complex_t(m8[4], m8[5]), complex_t(m8[6], m8[7]));
        run(Rot_Bool(reg, digit, m), *static_cast<State*>(h), c, dag != 0);
    })
}
int ref_condrot(void* h, uint32_t reg_in, uint32_t reg_out, int dag, const sq_cond* c) {
    REF_TRY(run(CondRot_Rational_Bool(reg_in, reg_out), *static_cast<State*>(h), c, dag != 0))
}
int ref_condrot_general(void* h, uint32_t reg_in, uint32_t reg_out, const double* table, uint64_t n_values,
                        const sq_cond* c) {
    REF_TRY({
        std::vector<u22_t> t(n_values);
        for (uint64_t v = 0; v < n_values; ++v) {
            const double* m = table + 8 * v;
            t[v] = u22_t(complex_t(m[0], m[1]), complex_t(m[2], m[3]), complex_t(m[4], m[5]), complex_t(m[6], m[7]));
        }
        auto f = [&t](uint64_t v) { return t.at(v); };
        run(CondRot_General_Bool_Fast<decltype(f)>(reg_in, reg_out, f), *static_cast<State*>(h), c, false);
    })
}
int ref_clear_zero(void* h, double eps) {
    REF_TRY({
        const ClearZero cz(eps);
        cz(*static_cast<State*>(h));
    })
}
int ref_normalize(void* h) {
    REF_TRY({
        const Normalize nz;
        nz(*static_cast<State*>(h));
    })
}
int ref_split_register(void* h, uint32_t first, uint32_t size, uint32_t* id) {
    REF_TRY({
        *id = (uint32_t)SplitRegister(first, "s" + std::to_string(g_names++), size)(
            *static_cast<State*>(h));
    })
}
int ref_combine_register(void* h, uint32_t first, uint32_t second) {
    REF_TRY(CombineRegister(first, second)(*static_cast<State*>(h)))
}

}  // extern "C"
