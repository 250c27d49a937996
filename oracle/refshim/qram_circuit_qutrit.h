// qram_circuit_qutrit.h — TEST INFRASTRUCTURE ONLY (oracle/). A minimal
// stand-in for the header of the reference's absent git submodule
// extern/qram-simulator, so that the reference's own CPU sources
// (SparQ/src/*.cpp) compile here, unmodified, into oracle/_ref/ and pin the
// oracle. Every helper is restated from how the SparQ sources use it, with the
// same semantics the oracle (sparq_oracle.cpp) assumes for it:
//   pow2(n)           2^n as a 64-bit word (0 for n >= 64)
//   width_mask(w)     low-w-bit mask, all ones for w >= 64
//                     (spelled out at quantum_arithmetic.cpp:332)
//   get_complement    two's-complement value of a w-bit field
//   epsilon           1e-14 (clearzero_default_eps, system_operations.h:577)
//   sqrt2inv          correctly rounded 1/sqrt(2)
//   sort_merge_unique_erase  a stable sort by the order given, each run of
//                     equal entries merged into its first in order, then the
//                     entries the predicate marks removed erased
// The noisy-QRAM machinery (branches, damping) is not restated: the pinned
// QRAMLoad is the noise-free load, QRAMCircuit::is_noise_free() is true.
// This header is not the submodule's and holds none of its code.
#pragma once

#include <algorithm>
#include <cmath>
#include <complex>
#include <cstddef>
#include <cstdint>
#include <execution>
#include <fstream>
#include <functional>
#include <iostream>
#include <regex>
#include <filesystem>
#include <map>
#include <random>
#include <set>
#include <sstream>
#include <stdexcept>
#include <string>
#include <string_view>
#include <tuple>
#include <type_traits>
#include <utility>
#include <vector>

#ifndef HOST_DEVICE
#define HOST_DEVICE
#endif

// ---------------------------------------------------------------- fmt (formatting only)
// The SparQ sources format strings for printing and error messages; the pin
// never reads them, so format() keeps the format string and the arguments
// are dropped.
namespace fmt {
template <typename... Args>
inline std::string format(std::string_view f, Args&&...) { return std::string(f); }
template <typename... Args>
inline void print(Args&&...) {}
}  // namespace fmt

namespace qram_simulator {

using complex_t = std::complex<double>;

// register kinds (an unscoped enum: the sources name the members bare; the
// pinned code compares them, it never reads their numbers)
enum StateStorageType { General, UnsignedInteger, SignedInteger, Boolean, Rational };

inline constexpr double pi = 3.14159265358979323846;
inline constexpr double epsilon = 1e-14;
inline const double sqrt2inv = 1.0 / std::sqrt(2.0);
inline const double sqrt2 = std::sqrt(2.0);

HOST_DEVICE constexpr inline uint64_t pow2(size_t n) { return n >= 64 ? 0 : (uint64_t{1} << n); }
HOST_DEVICE constexpr inline uint64_t width_mask(size_t w) { return w >= 64 ? ~uint64_t{0} : pow2(w) - 1; }
inline double abs_sqr(const complex_t& a) { return a.real() * a.real() + a.imag() * a.imag(); }
inline double abs_sqr(double a) { return a * a; }
inline bool ignorable(double v, double threshold = epsilon) { return std::abs(v) < threshold; }

HOST_DEVICE inline int64_t get_complement(uint64_t v, size_t size) {
    if (size == 0) return 0;
    if (size >= 64) return (int64_t)v;
    if ((v >> (size - 1)) & 1) return (int64_t)(v - pow2(size));
    return (int64_t)v;
}
HOST_DEVICE inline uint64_t make_complement(int64_t v, size_t size) { return (uint64_t)v & width_mask(size); }
// the digit-th bit of v
HOST_DEVICE inline uint64_t get_digit(uint64_t v, size_t digit) { return (v >> digit) & 1; }
template <typename T>
HOST_DEVICE inline T flip_digit(T v, size_t digit) { return v ^ (T(1) << digit); }
HOST_DEVICE inline bool digit1(uint64_t v, size_t digit) { return (v >> digit) & 1; }
HOST_DEVICE inline bool digit0(uint64_t v, size_t digit) { return !((v >> digit) & 1); }
HOST_DEVICE inline int bitcount(uint64_t v) { return __builtin_popcountll(v); }
HOST_DEVICE inline bool bit_parity(uint64_t v) { return __builtin_popcountll(v) & 1; }
// a fraction in [0, 1) as a size-bit word, truncated (a NaN gives 0: the
// conversion of a NaN is undefined in C++)
inline uint64_t get_rational(double x, size_t size) {
    if (std::isnan(x)) return 0;
    return (uint64_t)(x * (double)pow2(size)) & width_mask(size);
}
inline std::string dec2bin(uint64_t v, size_t size) {
    std::string s(size, '0');
    for (size_t i = 0; i < size; ++i)
        if ((v >> i) & 1) s[size - 1 - i] = '1';
    return s;
}
// floor(sqrt(v)), bit by bit
inline uint64_t isqrt_u64(uint64_t v) {
    uint64_t r = 0, bit = uint64_t{1} << 62;
    while (bit > v) bit >>= 2;
    while (bit) {
        if (v >= r + bit) {
            v -= r + bit;
            r = (r >> 1) + bit;
        } else {
            r >>= 1;
        }
        bit >>= 2;
    }
    return r;
}
// the value of the concatenated fields (v0 lowest, each field its own width)
inline size_t concat_value(const std::vector<std::pair<size_t, size_t>>& vw) {
    size_t out = 0, shift = 0;
    for (auto& [v, w] : vw) {
        out |= (v & width_mask(w)) << shift;
        shift += w;
    }
    return out;
}

// ---------------------------------------------------------------- errors
template <typename... Args>
[[noreturn]] inline void throw_invalid_input(Args&&...) { throw std::invalid_argument("invalid input"); }
template <typename... Args>
[[noreturn]] inline void throw_general_runtime_error(Args&&...) { throw std::runtime_error("runtime error"); }
template <typename... Args>
[[noreturn]] inline void throw_bad_result(Args&&...) { throw std::runtime_error("bad result"); }
template <typename... Args>
[[noreturn]] inline void throw_not_implemented(Args&&...) { throw std::logic_error("not implemented"); }
template <typename... Args>
[[noreturn]] inline void throw_bad_switch_case(Args&&...) { throw std::logic_error("bad switch case"); }

// ---------------------------------------------------------------- misc
struct profiler {
    explicit profiler(std::string_view) {}
};

inline std::string get_type_str(StateStorageType t) {
    switch (t) {
        case General: return "General";
        case UnsignedInteger: return "UnsignedInteger";
        case SignedInteger: return "SignedInteger";
        case Boolean: return "Boolean";
        case Rational: return "Rational";
    }
    return "?";
}

// sorted and no two equal neighbours
template <typename T>
inline bool check_unique_sort(const std::vector<T>& v) {
    for (size_t i = 1; i < v.size(); ++i)
        if (!(v[i - 1] < v[i])) return false;
    return true;
}

template <typename Vec, typename Less, typename Eq, typename Merge, typename Remove>
inline void sort_merge_unique_erase(Vec& v, Less less, Eq eq, Merge merge, Remove remove) {
    std::stable_sort(v.begin(), v.end(), less);
    size_t w = 0;
    for (size_t i = 0; i < v.size();) {
        size_t j = i + 1;
        if (w != i) v[w] = v[i];
        while (j < v.size() && eq(v[w], v[j])) {
            merge(v[w], v[j]);
            ++j;
        }
        ++w;
        i = j;
    }
    v.resize(w);
    v.erase(std::remove_if(v.begin(), v.end(), remove), v.end());
}

// 0 .. n-1 and the Cartesian product of two ranges (debug printing)
inline std::vector<size_t> range(size_t n) {
    std::vector<size_t> r(n);
    for (size_t i = 0; i < n; ++i) r[i] = i;
    return r;
}
inline std::vector<std::pair<size_t, size_t>> product(const std::vector<size_t>& a, const std::vector<size_t>& b) {
    std::vector<std::pair<size_t, size_t>> r;
    for (auto x : a)
        for (auto y : b) r.emplace_back(x, y);
    return r;
}

struct random_engine {
    static std::mt19937_64& get_engine() {
        static std::mt19937_64 e(0);
        return e;
    }
    static void set_seed(uint64_t s) { get_engine().seed(s); }
    static double uniform01() { return std::uniform_real_distribution<double>(0.0, 1.0)(get_engine()); }
};

// 2x2 complex matrix {u00, u01, u10, u11}
struct u22_t {
    complex_t m[4]{};
    u22_t() = default;
    u22_t(complex_t a, complex_t b, complex_t c, complex_t d) : m{a, b, c, d} {}
    complex_t& operator[](size_t i) { return m[i]; }
    const complex_t& operator[](size_t i) const { return m[i]; }
    u22_t dagger() const { return u22_t(std::conj(m[0]), std::conj(m[2]), std::conj(m[1]), std::conj(m[3])); }
};

template <typename T>
struct DenseMatrix {
    size_t size = 0;
    std::vector<T> data;
    DenseMatrix() = default;
    explicit DenseMatrix(size_t n) : size(n), data(n * n) {}
    T& operator()(size_t i, size_t j) { return data[i * size + j]; }
    const T& operator()(size_t i, size_t j) const { return data[i * size + j]; }
};

}  // namespace qram_simulator

// ---------------------------------------------------------------- QRAM (noise free)
// The noisy-circuit types below only satisfy the declarations of qram.cpp's
// noisy branches; a noise-free QRAM never reaches them, and each throws.
namespace qram_simulator {
using memory_t = std::vector<uint64_t>;
enum class OperationType { Damping, Depolarizing };
inline constexpr int arch_qutrit = 0;
[[noreturn]] inline void noisy_qram_absent() { throw std::logic_error("noisy QRAM is not part of the pinned path"); }
struct TimeStep {
    template <typename... A>
    void append_noise_range_only(A&&...) { noisy_qram_absent(); }
    size_t last_step() const { noisy_qram_absent(); }
    template <typename... A>
    double _get_multiplier_impl_qutrit(A&&...) const { noisy_qram_absent(); }
    bool is_bad_branch(size_t) const { noisy_qram_absent(); }
};
struct BranchEntry {
    complex_t amplitude;
    uint64_t data_bus = 0;
};
struct BranchRef {
    size_t system_size() const { noisy_qram_absent(); }
    const BranchEntry* iterbeg() const { noisy_qram_absent(); }
};
struct QRAMBranch {
    static constexpr int arch_type = 0;
    size_t address = 0;
    double relative_multiplier = 1.0;
    BranchRef* good_ref = nullptr;
    QRAMBranch(size_t addr, size_t, size_t) : address(addr) {}
    bool is_good() const { noisy_qram_absent(); }
    size_t system_size() const { noisy_qram_absent(); }
    const BranchEntry* iterbeg() const { noisy_qram_absent(); }
};
namespace qram_qutrit {
// the data words of a QRAM of 2^address_size words of data_size bits
struct QRAMCircuit {
    size_t address_size = 0, data_size = 0;
    memory_t memory;
    std::vector<QRAMBranch> branches;
    std::vector<double> branch_probs;
    std::map<OperationType, double> noise_parameters;
    TimeStep time_step;
    QRAMCircuit() = default;
    QRAMCircuit(size_t a, size_t d) : address_size(a), data_size(d), memory(pow2(a), 0) {}
    QRAMCircuit(size_t a, size_t d, memory_t mem) : address_size(a), data_size(d), memory(std::move(mem)) {}
    bool is_noise_free() const { return true; }
    bool has_damping() const { return false; }
    std::vector<QRAMBranch>& get_branches() { return branches; }
    std::vector<double>& get_branch_probs() { return branch_probs; }
    void run(std::string_view) { noisy_qram_absent(); }
    void sample_output_without_normalization() { noisy_qram_absent(); }
};
}  // namespace qram_qutrit
}  // namespace qram_simulator
