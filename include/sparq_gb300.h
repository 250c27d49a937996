/*
 * sparq_gb300.h — C ABI of the GB300 (sm_103a) engine for SparQ's sparse-state
 * gate-application path.
 *
 * The engine keeps a sparse quantum state in HBM as structure-of-arrays:
 *   - K packed 64-bit key words per basis entry (every active register is a bit
 *     field of width <= 64 inside one word; word-major arrays, one per word);
 *   - one complex128 amplitude per entry (interleaved re/im, 16 bytes).
 *
 * Every entry point returns an sq_status (0 = success). No C++ exception crosses
 * this boundary; sq_last_error() returns a message for the last failure on the
 * calling thread. All calls are stream-ordered on the library's stream and are
 * synchronous with respect to the host where they return sizes.
 *
 * Each declaration cites the reference interface it replaces (paths are relative
 * to the SparQSim project root). Register ids, condition kinds, XOR-out
 * conventions and the order of matrix elements follow the reference operators.
 */
#ifndef SPARQ_GB300_H
#define SPARQ_GB300_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define SQ_ABI_VERSION 1
#define SQ_MAX_REGISTERS 64     /* same cap as the reference CUDA build (basic_components.h:223-236) */
#define SQ_MAX_KEY_WORDS 8      /* 512 packed key bits per entry */
#define SQ_MAX_CONDITIONS 8
#define SQ_MAX_PROGRAM 32       /* instructions per fused elementwise launch */

typedef enum {
    SQ_OK = 0,
    SQ_ERR_INVALID = 1,        /* bad argument (reference: throw_invalid_input) */
    SQ_ERR_CUDA = 2,           /* CUDA runtime error (reference: CUDA_CHECK) */
    SQ_ERR_OOM = 3,            /* device allocation failed */
    SQ_ERR_CAPACITY = 4,       /* a size exceeds a documented maximum */
    SQ_ERR_DEVICE_TIMEOUT = 5, /* a bounded device-side wait gave up */
    SQ_ERR_BAD_RESULT = 6,     /* NaN norm (reference: throw_bad_result, dark_magic.cpp:26-27) */
    SQ_ERR_UNSUPPORTED = 7,    /* operation/shape not provided by this engine */
    SQ_ERR_NO_DEVICE = 8       /* no CUDA device visible */
} sq_status;

/* Register types; reference StateStorageType (qram-simulator submodule). */
typedef enum {
    SQ_GENERAL = 0,
    SQ_UNSIGNED = 1,
    SQ_SIGNED = 2,
    SQ_BOOLEAN = 3,
    SQ_RATIONAL = 4
} sq_reg_type;

/* Control conditions, AND-combined; reference ClassControllable
 * (global_macros.h:28-86, 104-284). */
typedef enum {
    SQ_COND_NONZERO = 0,  /* register value != 0            (conditioned_by_nonzeros) */
    SQ_COND_ALL_ONES = 1, /* register value == 2^width - 1  (conditioned_by_all_ones) */
    SQ_COND_BIT = 2,      /* bit `param` of register is 1   (conditioned_by_bit)      */
    SQ_COND_VALUE = 3     /* register value == param         (conditioned_by_value)    */
} sq_cond_kind;

typedef struct {
    uint32_t kind;   /* sq_cond_kind */
    uint32_t reg;    /* register id */
    uint64_t param;  /* bit position (SQ_COND_BIT) or value (SQ_COND_VALUE) */
} sq_condition;

typedef struct {
    uint32_t count;  /* number of valid entries in c[] */
    uint32_t reserved;
    sq_condition c[SQ_MAX_CONDITIONS];
} sq_cond;

/* Elementwise opcodes. Each is one reference operator's per-entry update;
 * the comment gives the reference (file:line of the CPU loop) and the
 * operand slots used in sq_instr (reg[0..3], imm[0..2], c[0..7]). */
typedef enum {
    SQ_OP_NOP = 0,
    SQ_OP_FLIP_BOOLS = 1,            /* quantum_arithmetic.cpp:11-30   reg0 = ~reg0 & mask */
    SQ_OP_SWAP_BOOL_BOOL = 2,        /* :32-61    reg0 bit imm0 <-> reg1 bit imm1 */
    SQ_OP_SHIFT_LEFT = 3,            /* :63-92    cyclic rotate reg0 left by imm0 */
    SQ_OP_SHIFT_RIGHT = 4,           /* :95-121   cyclic rotate reg0 right by imm0 */
    SQ_OP_MULT_UINT_CONST = 5,       /* :137-155  reg2 = (reg2 ^ reg0*imm0) & mask(reg2) */
    SQ_OP_ADD_MULT_UINT_CONST = 6,   /* :157-196  reg2 = (reg2 +/- imm0*reg0) & mask */
    SQ_OP_MOD_MULT_CONST = 7,        /* :222-285  reg0 = reg0*imm0 % imm1 (imm0 = opnum) */
    SQ_OP_ADD_UINT_UINT = 8,         /* :287-306  reg2 ^= (reg0 + reg1) & mask */
    SQ_OP_ADD_UINT_UINT_INPLACE = 9, /* :308-349  reg1 = (reg1 +/- reg0) & mask */
    SQ_OP_ADD_UINT_CONST = 10,       /* :351-369  reg2 ^= (reg0 + imm0) & mask */
    SQ_OP_ADD_CONST_INPLACE = 11,    /* :371-411  reg0 = (reg0 +/- imm0) & mask */
    SQ_OP_SUB_UINT_UINT = 12,        /* :490-509  reg2 ^= (reg0 - reg1) & mask */
    SQ_OP_NEG_UINT = 13,             /* :511-530  reg1 ^= (0 - reg0) & mask */
    SQ_OP_ABS_SINT = 14,             /* :532-554  reg1 ^= |sext(reg0)| & mask */
    SQ_OP_MUL_UINT_UINT = 15,        /* :556-575  reg2 ^= (reg0 * reg1) & mask */
    SQ_OP_DIV_UINT_UINT = 16,        /* :577-600  reg2 ^= (reg1 ? reg0/reg1 : 0) & mask */
    SQ_OP_SQRT_UINT = 17,            /* :602-620  reg1 ^= isqrt(reg0) & mask */
    SQ_OP_SELECT_BOOL = 18,          /* :623-644  reg3 ^= (reg0&1 ? reg1 : reg2) & mask */
    SQ_OP_AND_UINT_UINT = 19,        /* :646-665 */
    SQ_OP_OR_UINT_UINT = 20,         /* :667-686 */
    SQ_OP_XOR_UINT_UINT = 21,        /* :688-707 */
    SQ_OP_LESS_SINT_SINT = 22,       /* :709-729  reg2 ^= sext(reg0) < sext(reg1) */
    SQ_OP_CARRY_UINT_UINT = 23,      /* :731-754  reg3 ^= carry out of width(reg2) */
    SQ_OP_OVERFLOW_SINT_SINT = 24,   /* :756-785  reg3 ^= signed overflow at width(reg2) */
    SQ_OP_MULOVERFLOW_UINT_UINT = 25,/* :787-817  reg3 ^= product overflows width(reg2) */
    SQ_OP_ISZERO_UINT = 26,          /* :819-837  reg1 ^= (reg0 == 0) */
    SQ_OP_NEGATIVE_SINT = 27,        /* :839-857  reg1 ^= sext(reg0) < 0 */
    SQ_OP_ADD_ANYINT_INPLACE = 28,   /* :869-907  reg0 = (reg0 +/- ext(reg1)) & mask(reg0) */
    SQ_OP_ASSIGN = 29,               /* :909-930  reg1 = (reg1 ^ reg0) & mask(reg1) */
    SQ_OP_COMPARE_UINT_UINT = 30,    /* :932-959  eq: reg3 ^= 1, else reg2 ^= (l < r) */
    SQ_OP_LESS_UINT_UINT = 31,       /* :961-980  reg2 ^= (reg0 < reg1) */
    SQ_OP_SWAP_GENERAL = 32,         /* :982-999  swap(reg0, reg1) */
    SQ_OP_GETMID_UINT_UINT = 33,     /* :1001-1020 reg2 ^= (reg0 + reg1) / 2 */
    SQ_OP_X_BOOL = 34,               /* basic_gates.cpp:383-401  flip bit imm0 of reg0 */
    SQ_OP_INIT_UNSAFE = 35,          /* dark_magic.cpp:35-40     reg0 = imm0 */
    SQ_OP_QRAM_LOAD = 36,            /* qram.cpp:15-35  reg1 ^= table[reg0 mod 2^addr_size] */
    SQ_OP_PLUS_ONE_OVERFLOW = 37,    /* SparQ_Algorithm/src/BlockEncoding/block_encoding_tridiagonal.cpp:20-83
                                        reg0 = reg0 +/- 1 mod 2^width; on the wrap reg1 = (reg1 + 1) % 2 */
    /* A bit permutation of one register (no single reference operator; the
     * index map of Hadamard_Partial, map_position / from_map_position,
     * hadamard.cpp:443-466): imm0 = a set of bit positions (a mask below the
     * register's width); dag = 0 moves those bits, in ascending order, to
     * the lowest bits and the other bits, in order, above them; dag = 1
     * moves them back. */
    SQ_OP_BIT_GATHER = 38,
    /* amplitude-only or key+amplitude elementwise ops */
    SQ_OP_PHASE_BOOL = 64,           /* basic_gates.cpp:11-54  amp *= c0 if bit imm0 of reg0 */
    SQ_OP_GLOBAL_PHASE = 65,         /* parallel_phase_operations.cpp:72-107  amp *= c0 */
    SQ_OP_Y_BOOL = 66,               /* basic_gates.cpp:418-441 */
    SQ_OP_REFLECTION_BOOL = 67,      /* parallel_phase_operations.cpp:46-70 imm0 = bitmask of register ids, imm1 = inverse */
    SQ_OP_ZERO_COND_PHASE_FLIP = 68, /* parallel_phase_operations.cpp:11-31 imm0 = bitmask of register ids */
    SQ_OP_ROT_DIAGONAL = 69,         /* basic_gates.cpp:110-133 amp *= (bit ? c1 : c0) */
    SQ_OP_ROT_OFF_DIAGONAL = 70,     /* basic_gates.cpp:146-171 flip bit, amp *= (bit ? c1 : c0) */
    /* Per-trajectory Pauli noise for batched trajectories (no single reference
     * operator; equivalent to X_Bool / Z_Bool conditioned_by_value on the
     * trajectory register): t = reg0; if t < imm0, with masks
     * w[6t .. 6t+5] = (xa, xb, xc, za, zb, zc) read from `qram`:
     * reg1 ^= xa, reg2 ^= xb, reg3 ^= xc, then
     * amp *= (-1)^(popcount(reg1 & za) + popcount(reg2 & zb) + popcount(reg3 & zc)). */
    SQ_OP_PAULI_NOISE = 71,
    /* The CKS walk on a constant-diagonal tridiagonal matrix with 4-slot row
     * windows (SparQ_Algorithm/include/hamiltonian_simulation_tridiagonal.h:
     * 104-190). mem(idx) is the word of the combined [elements | columns]
     * table at idx & (8n - 1); imm0 = n (a power of two >= 8), imm1 =
     * alpha_enc | beta_enc << 32 (the quantised elements, < 2^32 each).
     * TridiagOracle1 (hamiltonian_tridiagonal.cpp:16-33):
     *   reg3 ^= mem(reg0 + 4 * reg1 + reg2)  (offset, row, slot, data). */
    SQ_OP_TRIDIAG_ELEMENT = 72,
    /* TridiagOracle2 (hamiltonian_tridiagonal.cpp:35-83) on offset reg0,
     * row reg1, slot/column reg2 and tag reg3, imm2 = k_width; dag = 0 maps
     * column -> slot, dag = 1 slot -> column. The tag is read modulo
     * 2^k_width; the dagger stores it unmasked, so it wants a register wide
     * enough for row addresses (64 bits) to keep every bit the reference
     * keeps. */
    SQ_OP_TRIDIAG_SLOT_COLUMN = 73,
    /* reg1 ^= f(reg0), f from a table of sq_lookup_create (passed in `qram`);
     * a value the table does not hold XORs 0 and is reported as
     * SQ_ERR_INVALID at the next synchronising call. */
    SQ_OP_LOOKUP_XOR = 74,
    /* TridiagParityPhase (hamiltonian_tridiagonal.cpp:88-105): amp = -amp
     * where reg0 is odd. */
    SQ_OP_PARITY_PHASE = 75,
    /* reg2 ^= angle(reg0, reg1), the rational angle word of imm0's operator
     * (SQ_ANGLE_*) looked up in a table of sq_angle_table_create (passed in
     * `qram`): Div_Sqrt_Arccos_UInt_UInt (quantum_arithmetic.cpp:413-432) or
     * GetRotateAngle_Int_Int (quantum_arithmetic.cpp:458-487). A pair the
     * table does not hold XORs 0 and is reported as SQ_ERR_INVALID at the
     * next synchronising call. */
    SQ_OP_ANGLE_XOR = 76,
    /* The address arithmetic of the sparse-matrix oracles:
     * reg3 ^= reg0 + imm0 * reg1 (+ reg2 when imm1 = 1), the sum in 64 bits,
     * XORed into reg3 within its width: GetRowAddr (imm1 = 0) and GetDataAddr
     * (imm1 = 1), SparQ_Algorithm/src/hamiltonian_simulation.cpp:222-253. */
    SQ_OP_ADDR_XOR = 77,
    /* QuantumBinarySearch_Fast (hamiltonian_simulation.cpp:182-220): with the
     * QRAM table in `qram`, l = reg0, r = l + imm0, imm1 rounds of
     * mid = (l + r) / 2 compared with reg1 (equal: the result is mid; word <
     * target: l = mid, else r = mid); reg2 ^= the result (0 when not found).
     * Addresses are taken modulo the table's size. */
    SQ_OP_QBS_XOR = 78
} sq_opcode;

/* One elementwise instruction. Register ids in reg[], integer constants in
 * imm[], complex constants as (re, im) pairs in c[]. `dag` selects the
 * inverse for in-place ops that have one. */
typedef struct sq_qram sq_qram;
typedef struct {
    uint32_t op;        /* sq_opcode */
    uint32_t dag;       /* 1 = apply the adjoint (in-place arithmetic) */
    uint32_t reg[4];
    uint64_t imm[3];
    double c[8];        /* c0 = (c[0], c[1]), c1 = (c[2], c[3]), ... */
    const sq_qram* qram;
    sq_cond cond;
} sq_instr;

typedef struct sq_state sq_state;

/* ------------------------------------------------------------------ */
/* Library                                                            */
/* ------------------------------------------------------------------ */
int sq_abi_version(void);
const char* sq_last_error(void);
/* Select the CUDA device and create the library stream (idempotent). */
int sq_init(int device);
/* Block until all work on the library stream is done; reports device-side
 * error flags raised by bounded waits (SQ_ERR_DEVICE_TIMEOUT). */
int sq_synchronize(void);
/* The number of polls after which every bounded device-side wait gives up
 * (decoupled look-backs of ClearZero, group starts, count scans and the radix
 * sort's per-digit look-back; the hash grouping's wait on a locked slot): the
 * waiting block raises the device error word, finishes without waiting
 * further, and the next synchronising call returns SQ_ERR_DEVICE_TIMEOUT.
 * 0 restores the default, 2^22 polls. Stream-ordered: launches already
 * queued keep the limit they were queued with. No counterpart in the
 * reference, whose kernels have no waits between blocks. */
int sq_set_wait_limit(uint32_t polls);
int sq_get_wait_limit(uint32_t* polls);
/* Exercises that failure path: one ClearZero look-back (two tiles of zero
 * amplitudes in library scratch, one block) whose predecessor tile is never
 * published, with a limit of `polls` (1..2^20). Returns SQ_ERR_DEVICE_TIMEOUT
 * when the wait gave up and was reported as it must be, and leaves the
 * library usable; SQ_OK would mean the wait did not end as specified. */
int sq_selftest_wait_timeout(uint32_t polls);
/* Number of device allocations (cudaMalloc, cudaMallocAsync) this library
 * has made since load; callers that must not see the library allocate can
 * check that a call left it unchanged. */
int sq_device_allocation_count(uint64_t* count);
/* Number of kernels this library has launched since load. */
int sq_launch_count(uint64_t* count);
/* The library's CUDA stream (cudaStream_t), for callers that order their own work after it. */
int sq_get_stream(void** stream);
/* Per-kernel device timing (no counterpart in the reference, which times
 * whole operators with std::chrono): while enabled, every launch is bracketed
 * by CUDA events on the library stream. sq_profile_read copies up to `max`
 * kernels: NUL-separated names into names_buf, launch counts, total ms and the
 * total algorithmic (compulsory) HBM bytes of those launches. */
int sq_profile_enable(int on);
int sq_profile_reset(void);
int sq_profile_read(char* names_buf, size_t buf_len, uint64_t* counts, double* total_ms, double* total_bytes,
                    uint32_t max, uint32_t* n_out);

/* ------------------------------------------------------------------ */
/* Register table — process-global, like System::name_register_map     */
/* (basic_components.h:239-283, basic_components.cpp:151-459).        */
/* ------------------------------------------------------------------ */
/* System::clear (basic_components.cpp:151-163) */
int sq_system_clear(void);
/* System::add_register (basic_components.cpp:330-364): reuses freed ids LIFO. */
int sq_system_add_register(uint32_t type, uint32_t width, uint32_t* id_out);
/* System::remove_register (basic_components.cpp:378-389) */
int sq_system_remove_register(uint32_t id);
/* System::type_of / size_of / status_of plus this engine's packing. */
int sq_system_register_info(uint32_t id, uint32_t* type, uint32_t* width, uint32_t* active,
                            uint32_t* word, uint32_t* shift);
int sq_system_register_count(uint32_t* n);
int sq_system_key_words(uint32_t* k);
int sq_system_set_register_type(uint32_t id, uint32_t type);

/* ------------------------------------------------------------------ */
/* State — replaces CuSparseState (cuda/basic_components.cuh:161-328). */
/* ------------------------------------------------------------------ */
/* A new state holds one entry |0...0> with amplitude 1 (SparseState(),
 * basic_components.h:604-606). `capacity` is an initial reservation. */
int sq_state_create(uint64_t capacity, sq_state** out);
int sq_state_destroy(sq_state* st);
int sq_state_size(const sq_state* st, uint64_t* n);
int sq_state_capacity(const sq_state* st, uint64_t* cap);
int sq_state_reserve(sq_state* st, uint64_t capacity);
/* reset_systems (system_operations.cpp:107-116): one zero entry, amplitude 1. */
int sq_state_reset(sq_state* st);
int sq_state_copy(sq_state* dst, const sq_state* src);
/* Host AoS upload/download, one uint64 per register id per entry (the
 * reference System layout): regs[i * nregs + id], amps[2*i], amps[2*i+1]. */
int sq_state_upload(sq_state* st, uint64_t n, const uint64_t* regs, uint32_t nregs, const double* amps);
int sq_state_download(const sq_state* st, uint64_t* regs, uint32_t nregs, double* amps);
/* Packed transfer in the engine's own layout: keys[w * n + i] for w < K
 * (K from sq_system_key_words), amps[2*i], amps[2*i+1]. No per-register
 * packing on the host, so these run at copy bandwidth (CuSparseState
 * move_to_gpu / copy_to_cpu, cuda/basic_components.cu:49-106). */
int sq_state_upload_packed(sq_state* st, uint64_t n, const uint64_t* keys, const double* amps);
int sq_state_download_packed(const sq_state* st, uint64_t* keys, double* amps);
/* The same download, enqueued behind the work already queued on the library
 * stream and returned from at once, so that it overlaps later work on other
 * states. The host buffers must stay valid until sq_state_wait(st) (or
 * sq_synchronize) returns; a later call that writes or frees this state
 * waits for the copy on the device first. */
int sq_state_download_packed_async(sq_state* st, uint64_t* keys, double* amps);
/* Blocks until the state's last asynchronous download has finished. */
int sq_state_wait(sq_state* st);
/* How asynchronous downloads into pinned host memory are moved:
 * SQ_DOWNLOAD_SM_STORES (default) by a few low-priority blocks storing over
 * the host link (about 150 GB/s, steady from one system to the next), so that
 * the small count reads of eagerly issued operators are not queued behind a
 * bulk transfer; SQ_DOWNLOAD_COPY_ENGINE by the copy engine, which takes no
 * SM resources from the work it overlaps (graph replays read no counts back)
 * but whose rate into pinned memory was measured from 84 to over 170 GB/s on
 * different systems. Other host memory always goes by the copy engine. */
#define SQ_DOWNLOAD_SM_STORES 0
#define SQ_DOWNLOAD_COPY_ENGINE 1
/* Both at once: the first half of each pinned destination by SM stores, the
 * second by the copy engine. */
#define SQ_DOWNLOAD_SPLIT 2
int sq_set_download_engine(int engine);

/* ------------------------------------------------------------------ */
/* Graphs: a sequence of operators replayed as one CUDA graph launch    */
/* ------------------------------------------------------------------ */
/* 1. sq_graph_record_begin(st); apply the operators to the state (they run
 *    eagerly; every count the host reads back is logged); sq_graph_record_end().
 *    The sequence must leave the state's double buffers in their roles (an
 *    even number of splits), so that every replay starts as the last ended. 
 * 2. Bring the state back to the same input (the same size, e.g. upload it
 *    again), then sq_graph_capture_begin(st); apply the same operators (they
 *    are captured, not run, and take the logged counts); sq_graph_capture_end.
 * 3. For every replay: bring the state to the same input and call
 *    sq_graph_launch. Every count, offset and size in the graph was recorded
 *    for one input, so a launch is refused (SQ_ERR_INVALID, before anything
 *    runs) unless the state's entries and the content of every table the
 *    operators read (QRAM, lookup, noise) have the checksums they had when
 *    recorded, and the state's buffers and the library's workspace are those
 *    captured; the checksums cost one reduction and one synchronisation. The
 *    logged counts are also checked on the device (a mismatch is reported as
 *    SQ_ERR_INVALID at the next synchronising call). A launch after the state
 *    or a table the operators read was destroyed is refused on the host
 *    (SQ_ERR_INVALID) before any device work. Allocation is refused while
 *    capturing: the record pass grows every buffer. */
typedef struct sq_graph sq_graph;
int sq_graph_record_begin(sq_state* st);
int sq_graph_record_end(void);
int sq_graph_capture_begin(sq_state* st);
int sq_graph_capture_end(sq_graph** out);
int sq_graph_launch(sq_graph* g);
int sq_graph_destroy(sq_graph* g);
/* Diagnostics: the captured graph as a DOT file with every node's parameters
 * (cudaGraphDebugDotPrint, verbose), and a text listing of a state's buffers,
 * group-range sets and the library's workspace slots. */
int sq_graph_debug_dot(const sq_graph* g, const char* path);
int sq_state_debug_layout(const sq_state* st, char* buf, uint64_t len);
/* Device pointers of the live arrays (valid until the next call that resizes). */
int sq_state_device_arrays(sq_state* st, uint64_t** key_words, uint32_t* k, double** amps);

/* ------------------------------------------------------------------ */
/* QRAM table — replaces CuQRAMCircuit::memory_dev (cuda/qram.cu:68-107) */
/* ------------------------------------------------------------------ */
/* qram_qutrit::QRAMCircuit(addr_size, data_size, memory): the table has
 * 2^address_size words; it is copied to HBM once, narrowed to the smallest
 * of u16/u32/u64 that holds every word. */
int sq_qram_create(uint32_t address_size, uint32_t data_size, const uint64_t* memory, uint64_t n_words,
                   sq_qram** out);
/* New words for an existing table (2^address_size of them), written in place
 * on the library stream: launches queued or captured earlier keep reading the
 * same device table. The words must fit the width the table was stored at
 * (that of the words it was created with); otherwise SQ_ERR_INVALID and the
 * table keeps its previous content (the words are checked before any is
 * written). */
int sq_qram_write(sq_qram* q, const uint64_t* memory, uint64_t n_words);
int sq_qram_destroy(sq_qram* q);
/* A classical function table for SQ_OP_LOOKUP_XOR: f(v) = dense[v] for
 * v < dense_len, words[i] for v == keys[i] (keys ascending, unique, each >=
 * dense_len). Released with sq_qram_destroy. */
int sq_lookup_create(const uint64_t* dense, uint64_t dense_len, const uint64_t* keys, const uint64_t* words,
                     uint64_t n_sparse, sq_qram** out);
/* The quantised walk angles of GetQWRotateAngle_Int_Int_Int
 * (SparQ_Algorithm/src/hamiltonian_simulation.cpp:257-291) for the element
 * values v[i]: ratio = v / (2^ds - 1) (positive_only) or
 * |sext(v)| / (2^(ds-1) - 1), clamped to [0, 1]; out[i] = the Rational
 * fixed point of acos(sqrt(ratio)) / (2 pi) at out_width bits (truncated).
 * Computed on the host with the C library's acos, so that the angles a
 * lookup table gives on the GPU are the CPU's bit for bit. */
int sq_qw_rotate_angle_words(const uint64_t* v, uint64_t n, uint32_t data_size, int positive_only,
                             uint32_t out_width, uint64_t* out);

/* Angle tables for SQ_OP_ANGLE_XOR. The reference computes these angles per
 * entry with the C library (acos, sqrt, atan2) and truncates them to a
 * Rational register (get_rational); a last-place difference in the device's
 * math functions would move a bit of the key, so the angles of the (lhs, rhs)
 * register pairs an operator can meet are computed here on the host with the
 * C library, exactly as the reference's CPU loop does, and looked up on the
 * GPU (an open-addressing hash, probes bounded by the longest insertion):
 *   SQ_ANGLE_DIV_SQRT_ARCCOS: acos(sqrt(lhs / rhs)) / (2 pi), unsigned values
 *     (Div_Sqrt_Arccos_UInt_UInt, quantum_arithmetic.h:1066);
 *   SQ_ANGLE_ROTATE: atan2(rhs, lhs) / (2 pi) in [0, 1) of the
 *     two's-complement values, 0.25 / 0.75 for lhs = 0 (GetRotateAngle_Int_Int,
 *     quantum_arithmetic.h:1266).
 * The word is the angle times 2^out_width, truncated; a NaN angle (0 / 0, or
 * lhs > rhs) gives 0 (the reference converts NaN to an integer, which C++
 * leaves undefined). Widths 1..63; pairs are taken modulo their widths and
 * repeats collapse. Released with sq_qram_destroy. */
#define SQ_ANGLE_DIV_SQRT_ARCCOS 0
#define SQ_ANGLE_ROTATE 1
int sq_angle_table_create(int kind, uint32_t lhs_width, uint32_t rhs_width, uint32_t out_width, const uint64_t* lhs,
                          const uint64_t* rhs, uint64_t n, sq_qram** out);
/* The word sq_angle_table_create stores for one pair (the host computation
 * itself, for callers that build their own tables). */
int sq_angle_word(int kind, uint32_t lhs_width, uint32_t rhs_width, uint32_t out_width, uint64_t lhs, uint64_t rhs,
                  uint64_t* word);

/* ------------------------------------------------------------------ */
/* Elementwise operators                                               */
/* ------------------------------------------------------------------ */
/* Runs up to SQ_MAX_PROGRAM instructions over every entry in one pass
 * (one launch); each instruction has its own conditions. */
int sq_apply_program(sq_state* st, const sq_instr* prog, uint32_t n);
/* Convenience entry points; each is a one-instruction program. */
int sq_add_uint_uint(sq_state* st, uint32_t lhs, uint32_t rhs, uint32_t res, const sq_cond* cond); /* Add_UInt_UInt, quantum_arithmetic.cpp:287 */
int sq_add_uint_uint_inplace(sq_state* st, uint32_t lhs, uint32_t rhs, const sq_cond* cond, int dag); /* :308,:327 */
int sq_add_uint_const(sq_state* st, uint32_t lhs, uint64_t c, uint32_t res, const sq_cond* cond); /* :351 */
int sq_add_const_inplace(sq_state* st, uint32_t reg, uint64_t c, const sq_cond* cond, int dag); /* :372,:392 */
int sq_mult_uint_const(sq_state* st, uint32_t lhs, uint64_t c, uint32_t res, const sq_cond* cond); /* :137 */
int sq_add_mult_uint_const(sq_state* st, uint32_t lhs, uint64_t c, uint32_t res, const sq_cond* cond, int dag); /* :157,:177 */
int sq_mul_uint_uint(sq_state* st, uint32_t lhs, uint32_t rhs, uint32_t res, const sq_cond* cond); /* :556 */
int sq_add_anyint_inplace(sq_state* st, uint32_t lhs, uint32_t rhs, const sq_cond* cond, int dag); /* :869,:889 */
int sq_assign(sq_state* st, uint32_t src, uint32_t dst, const sq_cond* cond); /* :909 */
int sq_shift(sq_state* st, uint32_t reg, uint32_t digits, int left, const sq_cond* cond); /* :63,:94 */
int sq_swap(sq_state* st, uint32_t a, uint32_t b, const sq_cond* cond); /* :981 */
int sq_x_bool(sq_state* st, uint32_t reg, uint32_t digit, const sq_cond* cond); /* basic_gates.cpp:383 */
int sq_flip_bools(sq_state* st, uint32_t reg, const sq_cond* cond); /* quantum_arithmetic.cpp:11 */
int sq_init_unsafe(sq_state* st, uint32_t reg, uint64_t value); /* dark_magic.cpp:35 */
/* QRAMLoad::noise_free_impl (qram.cpp:15-35): data ^= memory[addr mod 2^addr_size]. */
int sq_qram_load(sq_state* st, const sq_qram* q, uint32_t addr, uint32_t data, const sq_cond* cond);
/* Phase_Bool (basic_gates.cpp:11-54): amp *= e^{+-i lambda} where bit `digit` of reg is set. */
int sq_phase_bool(sq_state* st, uint32_t reg, uint32_t digit, double lambda, const sq_cond* cond, int dag);
/* GlobalPhase (parallel_phase_operations.cpp:72-107): amp *= c (conj(c) for dag). */
int sq_global_phase(sq_state* st, double re, double im, const sq_cond* cond, int dag);
/* Reflection_Bool (parallel_phase_operations.cpp:46-70). */
int sq_reflection_bool(sq_state* st, const uint32_t* regs, uint32_t nregs, int inverse, const sq_cond* cond);
/* ZeroConditionalPhaseFlip (parallel_phase_operations.cpp:11-31). */
int sq_zero_cond_phase_flip(sq_state* st, const uint32_t* regs, uint32_t nregs, const sq_cond* cond);

/* ------------------------------------------------------------------ */
/* Split / merge operators (group by key except target bits)           */
/* ------------------------------------------------------------------ */
/* Hadamard_Int (hadamard.cpp:18-162): H on the low n_digits bits of reg;
 * groups = entries equal on every other active bit; ClearZero(eps) after. */
int sq_hadamard_int(sq_state* st, uint32_t reg, uint32_t n_digits, const sq_cond* cond);
/* Batched Hadamard_Int: H on the low n bits of reg where n is each entry's
 * value of `width_reg` (n <= max_digits <= 8). Equivalent to applying
 * Hadamard_Int(reg, h).conditioned_by_value(width_reg, h) for every h, in one
 * pass; used to run trajectories of different widths in one state. */
int sq_hadamard_int_batched(sq_state* st, uint32_t reg, uint32_t width_reg, uint32_t max_digits, const sq_cond* cond);
/* Hadamard_Int_Full (hadamard.cpp:181-338): H on the whole register. */
int sq_hadamard_int_full(sq_state* st, uint32_t reg, const sq_cond* cond);
/* Hadamard_Bool (hadamard.cpp:340-439): reg must be 1 bit wide. */
int sq_hadamard_bool(sq_state* st, uint32_t reg, const sq_cond* cond);
/* Rot_Bool (basic_gates.cpp:74-357): 2x2 unitary mat = {m00, m01, m10, m11}
 * as 8 doubles (re, im) on bit `digit` of reg; dag applies mat^dagger. */
int sq_rot_bool(sq_state* st, uint32_t reg, uint32_t digit, const double* mat8, const sq_cond* cond, int dag);
/* CondRot_Rational_Bool (condrot.cpp:12-152): angle 2*pi*in/2^width(in) on the 1-bit out. */
int sq_condrot_rational_bool(sq_state* st, uint32_t reg_in, uint32_t reg_out, int dag);
/* The same applied to the entries that satisfy `cond` only, the others left as
 * they are: what the reference's composite operators (SPLIT_BY_CONDITIONS /
 * MERGE_BY_CONDITIONS, system_operations.h:109-129, around U_L and U_R in
 * block_encoding_via_QRAM.h:408-478) do to the CondRot inside them. */
int sq_condrot_rational_bool_cond(sq_state* st, uint32_t reg_in, uint32_t reg_out, int dag, const sq_cond* cond);
/* CondRot_General_Bool_Fast<F> (condrot.h:149-300): 2x2 unitary func(in) on
 * the 1-bit out register. The callable becomes a table: table[8*v .. 8*v+7]
 * = {m00, m01, m10, m11} as (re, im) for every v < 2^width(in) = n_values. */
int sq_condrot_general_bool(sq_state* st, uint32_t reg_in, uint32_t reg_out, const double* table, uint64_t n_values);
/* The same on the entries that satisfy `cond` only, the others left as they
 * are (the composite-operator form, as sq_condrot_rational_bool_cond): a walk
 * over a batch of problems rotates its ancilla by each problem's own matrix
 * under the problem's index, or by one matrix under the walk's conditions. */
int sq_condrot_general_bool_cond(sq_state* st, uint32_t reg_in, uint32_t reg_out, const double* table, uint64_t n_values,
                                 const sq_cond* cond);
/* Rot_GeneralUnitary (rot.cpp:353-477): dense dim x dim unitary (dim = 2^width(reg),
 * width <= 8) on the whole register, row-major (re, im) pairs; dag applies M^dagger. */
int sq_rot_general_unitary(sq_state* st, uint32_t reg, const double* mat, uint64_t dim, const sq_cond* cond, int dag);
/* Hadamard_Partial (hadamard.cpp:470-712): H on a set of bit positions of reg
 * (repeats collapse, as in the reference's std::set). One position: the
 * reference's active path (pairs of entries equal except that bit,
 * a*sqrt2inv +- b*sqrt2inv). Several: H on each bit of the set, as
 * Hadamard_Partial::operate over groups equal outside the set (hadamard.cpp:
 * 468-570), with the one-member sign (-1)^popcount(i & v) of the Hadamard
 * transform. Conditions are tested per entry (the reference's active path
 * ignores them). */
int sq_hadamard_partial(sq_state* st, uint32_t reg, const uint32_t* positions, uint32_t n_positions, const sq_cond* cond);

/* ------------------------------------------------------------------ */
/* Prune / norm / merge / register surgery                              */
/* ------------------------------------------------------------------ */
/* How split/merge operators group entries: 0 = automatic (hash grouping for
 * transforms on >= 4096 entries, sort otherwise; the add_systems merge always
 * sorts), 1 = onesweep radix sort, 2 = hash table. Results are identical;
 * only the entry order of the output differs. No counterpart in the reference
 * (its CPU path sorts or uses std::map buckets, its GPU path sorts). */
int sq_set_group_strategy(int strategy);
int sq_get_group_strategy(int* strategy);
/* Strategy 3 (the default) is autotuned: per shape class (operator kind,
 * conditions, key words, log2 N; 4096 entries and more) the first split runs
 * the sort grouping, the second the hash grouping, each timed around the
 * whole operator, and later splits of the class use the faster. */
int sq_autotune_reset(void);
int sq_autotune_classes(uint64_t* classes, uint64_t* decided);
/* How split operators size their output: 0 = automatic (one pass that
 * reserves each group's output range with an atomic, when the bound "every
 * group fully populated" fits in memory), 1 = exact count pass, scan, write
 * pass. Same entries either way; only their order differs. */
int sq_set_output_sizing(int mode);
int sq_get_output_sizing(int* mode);
/* Arithmetic of the Hadamard butterfly networks (Hadamard_Int, the full
 * buckets of Hadamard_Int_Full, Hadamard_Int_Batched):
 * SQ_ARITH_REFERENCE = FP64 butterflies (a0 +- a1) * sqrt2inv in the
 * reference's stage order (hadamard.cpp:44-59,100-131): bit-identical to the
 * reference's CPU results; SQ_ARITH_EXACT_SUM (the default) = each group's
 * amplitudes on one 64-bit integer grid, exact sums, one FP64 rounding per
 * output. Exact-sum results differ from the reference's by at most a few units
 * in the last place of the group's largest amplitude; keys are identical. It
 * exists because FP64 runs at a small fraction of the integer rate on GB300. */
enum { SQ_ARITH_REFERENCE = 0, SQ_ARITH_EXACT_SUM = 1 };

/* ------------------------------------------------------------------ size model
 * A learned model of split-operator output sizes (no counterpart in the
 * reference): a 3-layer FP32 MLP, SQ_PRED_FEATURES inputs -> 64 -> 64 -> 2,
 * ReLU, trained on the GPU by this library's own kernels on sizes logged by
 * the split operators. Features (per operator, before it runs): operator kind
 * one-hot [0..6] (Hadamard_Int, Hadamard_Int_Full, Hadamard_Bool, Rot_Bool,
 * CondRot, Rot_GeneralUnitary, merge), [7] per-entry width, [8] target
 * width / 16, [9] key words / 8, [10] log2 N / 32, [11] cached group ranges
 * usable, [12] log2(cached groups + 1) / 32, [13] conditions / 8, [15] 1, and
 * [16..47] a 32-register sketch (max leading-zero rank per hash bucket, / 32)
 * of the group keys of up to 65536 sampled entries. Outputs:
 * log2(groups / N) / 16 and log2((outputs + 1) / N) / 16. When enabled, the
 * predicted group count sizes the hash table and the predicted output count
 * gives a single-pass capacity where the fully populated bound is too large;
 * an overflow reruns the operator exactly, so results never depend on it.
 * Parameters are one float array: W1[48][64], b1[64], W2[64][64], b2[64],
 * W3[64][2], b3[2] (row-major, [in][out]). */
#define SQ_PRED_FEATURES 48
#define SQ_PRED_PARAMS 7426
int sq_predictor_reset(uint64_t seed);
int sq_predictor_get_params(float* out, uint64_t n);
int sq_predictor_set_params(const float* in, uint64_t n);
/* Mean-squared-error loss and its gradient (same layout as the parameters)
 * over n rows of features x[n][48] and targets t[n][2]; no update. */
int sq_predictor_gradient(const float* x, const float* t, uint64_t n, float* grad, float* loss);
int sq_predictor_predict(const float* x, uint64_t n, float* y);
/* Adam, `epochs` passes over n rows in shuffled minibatches of `batch`. */
int sq_predictor_train(const float* x, const float* t, uint64_t n, uint32_t epochs, uint32_t batch, float lr,
                       uint64_t seed, float* final_loss);
int sq_predictor_enable(int on);
/* Logging of (features, sizes) rows by the split operators (host memory). */
int sq_predictor_log_enable(int on);
int sq_predictor_log_size(uint64_t* rows);
int sq_predictor_log_read(float* x, float* t, uint64_t max_rows, uint64_t* rows);
int sq_predictor_log_clear(void);
/* Predictions made, and single passes that overflowed their capacity. */
int sq_predictor_stats(uint64_t* predictions, uint64_t* overflows);
/* Output entries a single-pass split may allocate by the fully populated
 * bound (a memory budget); 0 restores the default, max(4 N, 2^27). Beyond
 * it a split uses a predicted capacity, or else the exact count pass. */
int sq_set_single_pass_limit(uint64_t entries);
/* Groups the hash grouping's first table is sized for when no prediction is
 * made (default 2^20); more groups cost a second, larger attempt. */
int sq_set_hash_groups_hint(uint64_t groups);
int sq_set_fwht_arithmetic(int mode);
int sq_get_fwht_arithmetic(int* mode);
/* clearzero_default_eps (system_operations.h:577), initially 1e-14. */
int sq_set_clearzero_eps(double eps);
int sq_get_clearzero_eps(double* eps);
/* PartialTraceSelect (partial_trace.cpp:148-185): keep the entries whose
 * registers regs[i] hold values[i] (all i), in order, and scale them by
 * 1/sqrt(p), p their total probability; *result = that factor, +inf when
 * nothing is left, 0 for n == 0 or an empty state. The registers keep their
 * values. */
int sq_partial_trace_select(sq_state* st, const uint32_t* regs, const uint64_t* values, uint32_t n,
                            double* result);
/* PartialTraceSelectRange (partial_trace.cpp:187-225): the same for
 * lo <= value(reg) <= hi. */
int sq_partial_trace_select_range(sq_state* st, uint32_t reg, uint64_t lo, uint64_t hi, double* result);
/* GetOutput (SparQ_Algorithm qda_fundamental.cpp:123-166, the QDA read-out):
 * every entry whose registers zero_regs[] all hold 0 is placed in a dense
 * vector of 2^(sum of the widths of idx_regs) amplitudes at the index formed
 * by concatenating its idx_regs values, the first register in the lowest bits
 * (main + anc_1 * 2^n + anc_4 * 2^(n+1) for the QDA layout,
 * qda_fundamental.h:640-645); other slots are 0. *prob = those entries' total
 * probability; the vector is scaled by 1/sqrt(*prob) unless
 * |*prob - 1| < 1e-14 or *prob == 0. out (host memory) receives 2 doubles
 * (re, im) per slot, out_len slots, which must equal the vector length. The
 * zero and index registers together must cover every active register (so
 * that no two entries share a slot) and the index widths sum to at most 30;
 * otherwise SQ_ERR_INVALID. The state is unchanged. */
#define SQ_MAX_OUTPUT_FIELDS 8
int sq_get_output(sq_state* st, const uint32_t* zero_regs, uint32_t n_zero, const uint32_t* idx_regs,
                  uint32_t n_idx, double* out, uint64_t out_len, double* prob);
/* ClearZero (system_operations.cpp:371-382): drop entries with |a|^2 < eps;
 * order of survivors is preserved. */
int sq_clear_zero(sq_state* st, double eps);
/* ClearZero for callers that must not have the library allocate device
 * memory (programs that own every device buffer through their own pool or
 * framework allocator; loops where an implicit cudaMalloc, which may
 * synchronize the device, is not allowed). No counterpart in the reference.
 * Inputs and outputs are the caller's device arrays: k key-word arrays of n
 * words each plus n interleaved complex amplitudes in, the same layout out
 * (capacity >= n), survivor count to *n_out (host). The only scratch is a
 * fixed 262,400-byte static device array inside this library, so n is capped
 * at SQ_NOALLOC_MAX_ENTRIES; larger n returns SQ_ERR_CAPACITY. Work is issued
 * on `stream` (NULL = the default stream) and the call waits for it. The
 * first call on each device looks up that array's device address with the
 * device current; make that first call before capturing any stream. Under
 * CUDA's lazy module loading that first call is also when the driver places
 * the library's device code and the array in device memory, so device memory
 * in use can grow once there; later calls leave it unchanged. All calls
 * share the array: calls that overlap on the GPU race. No output array may
 * overlap an input array (blocks write outputs while others still read
 * inputs): overlapping arrays return SQ_ERR_INVALID. */
#define SQ_NOALLOC_MAX_ENTRIES (1ull << 26)
int sq_clear_zero_noalloc(const uint64_t* const* keys_in, const double* amps_in, uint32_t k, uint64_t n, double eps,
                          uint64_t* const* keys_out, double* amps_out, uint64_t* n_out, void* stream);
/* Normalize (dark_magic.cpp:11-32): a *= 1/sqrt(sum |a|^2); norm_sq_out may be NULL. */
int sq_normalize(sq_state* st, double* norm_sq_out);
/* Sum of |a|^2 (CheckNormalization's quantity, debugger.h). */
int sq_norm_sq(const sq_state* st, double* out);
/* add_systems (system_operations.h:157-175): dst += coef * src, entries with
 * equal keys summed, |a|^2 < eps dropped. */
int sq_add_systems(sq_state* dst, const sq_state* src, double coef);
/* AddRegister (system_operations.cpp:269-290): new zeroed register. */
/* AddRegisterWithHadamard (system_operations.cpp:281-305): a new register
 * of `width` bits, every entry copied 2^width times with the register taking
 * every value, amplitudes unchanged (no 2^(-width/2) factor, no prune). */
int sq_add_register_with_hadamard(sq_state* st, uint32_t type, uint32_t width, uint32_t* id_out);
int sq_add_register_sync(sq_state* st, uint32_t type, uint32_t width, uint32_t* id_out);
/* RemoveRegister / remove_register_synchronous (basic_components.cpp:398-430). */
int sq_remove_register_sync(sq_state* st, uint32_t id);
/* SplitRegister (system_operations.cpp:121-158): low `second_size` bits become a new register. */
int sq_split_register(sq_state* st, uint32_t first, uint32_t second_size, uint32_t* second_out);
/* CombineRegister (system_operations.cpp:165-203): first = first << |second| | second; second removed. */
int sq_combine_register(sq_state* st, uint32_t first, uint32_t second);

#ifdef __cplusplus
}
#endif
#endif /* SPARQ_GB300_H */
