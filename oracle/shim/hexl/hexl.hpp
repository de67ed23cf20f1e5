// hexl/hexl.hpp -- stand-in for the subset of the Intel HEXL API that the reference
// library calls.  TEST INFRASTRUCTURE ONLY: it exists so that the reference's own
// sources (yatfhe/src/*.cpp) can be compiled into the oracle under oracle/_ref/.
// HEXL itself is not installed here (and is x86-only); this file is written from the
// negacyclic-NTT mathematics in oracle/ntt_q.h, not from HEXL's code.
//
// API surface, with the reference call sites that fix its meaning:
//   NTT(degree, q), ComputeForward/ComputeInverse(out, in, 1, 1), GetModulus,
//   GetDegree, GetMinimalRootOfUnity     yatfhe/src/ntt_hexl.cpp:16-33,159,
//                                        yatfhe/include/yatfhe/ntt_hexl.h:34-44
//   EltwiseMultMod, EltwiseAddMod,       yatfhe/src/ntt_hexl.cpp:183-190,
//   EltwiseSubMod                        yatfhe/src/trgsw.cpp:456-524,
//                                        yatfhe/src/polynomial.cpp:411,420
//   AddUIntMod, SubUIntMod               yatfhe/src/polynomial.cpp:434,441,
//                                        yatfhe/src/blind_rotate.cpp:298-311
// Only input/output mod factors of 1 occur at those call sites (operands in [0, q)).
#ifndef YATFHE_ORACLE_HEXL_SHIM_HPP
#define YATFHE_ORACLE_HEXL_SHIM_HPP

#include <cstdint>
#include <cstring>
#include <memory>
#include <stdexcept>
#include <vector>

#include "../../ntt_q.h"

namespace intel {
namespace hexl {

class NTT {
public:
    NTT() = default;

    NTT(uint64_t degree, uint64_t q) : degree_(degree), q_(q), plan_(std::make_shared<Plan>()) {
        if (degree == 0 || (degree & (degree - 1)) != 0) {
            throw std::invalid_argument("NTT: degree must be a power of two");
        }
        if (nq_plan_init(&plan_->p, static_cast<uint32_t>(degree), q) != 0) {
            throw std::invalid_argument("NTT: modulus has no primitive 2N-th root of unity");
        }
    }

    void ComputeForward(uint64_t* result, const uint64_t* operand, uint64_t input_mod_factor,
                        uint64_t output_mod_factor) const {
        prepare(result, operand, input_mod_factor);
        nq_forward(&plan_->p, result);
        (void)output_mod_factor;  // results are always fully reduced to [0, q)
    }

    void ComputeInverse(uint64_t* result, const uint64_t* operand, uint64_t input_mod_factor,
                        uint64_t output_mod_factor) const {
        prepare(result, operand, input_mod_factor);
        nq_inverse(&plan_->p, result);
        (void)output_mod_factor;
    }

    uint64_t GetModulus() const { return q_; }
    uint64_t GetDegree() const { return degree_; }
    uint64_t GetMinimalRootOfUnity() const { return plan_ ? plan_->p.psi : 0; }

private:
    struct Plan {
        nq_plan p{};
        ~Plan() { nq_plan_free(&p); }
    };

    void prepare(uint64_t* result, const uint64_t* operand, uint64_t input_mod_factor) const {
        if (!plan_) throw std::logic_error("NTT: used before construction with (degree, q)");
        if (result != operand) std::memmove(result, operand, degree_ * sizeof(uint64_t));
        if (input_mod_factor != 1) {
            for (uint64_t i = 0; i < degree_; i++) result[i] %= q_;
        }
    }

    uint64_t degree_{0};
    uint64_t q_{0};
    std::shared_ptr<Plan> plan_{};
};

inline void EltwiseMultMod(uint64_t* result, const uint64_t* operand1, const uint64_t* operand2, uint64_t n,
                           uint64_t modulus, uint64_t input_mod_factor) {
    const nq_barrett br = nq_barrett_make(modulus);
    if (input_mod_factor == 1) {
        for (uint64_t i = 0; i < n; i++) result[i] = nq_mulmod(&br, operand1[i], operand2[i]);
    } else {
        for (uint64_t i = 0; i < n; i++) result[i] = nq_mulmod(&br, operand1[i] % modulus, operand2[i] % modulus);
    }
}

inline void EltwiseAddMod(uint64_t* result, const uint64_t* operand1, const uint64_t* operand2, uint64_t n,
                          uint64_t modulus) {
    for (uint64_t i = 0; i < n; i++) {
        uint64_t s = operand1[i] + operand2[i];
        result[i] = s >= modulus ? s - modulus : s;
    }
}

inline void EltwiseSubMod(uint64_t* result, const uint64_t* operand1, const uint64_t* operand2, uint64_t n,
                          uint64_t modulus) {
    for (uint64_t i = 0; i < n; i++) {
        result[i] = operand1[i] >= operand2[i] ? operand1[i] - operand2[i] : operand1[i] + modulus - operand2[i];
    }
}

inline uint64_t AddUIntMod(uint64_t x, uint64_t y, uint64_t modulus) {
    uint64_t s = x + y;
    return s >= modulus ? s - modulus : s;
}

inline uint64_t SubUIntMod(uint64_t x, uint64_t y, uint64_t modulus) {
    return x >= y ? x - y : x + modulus - y;
}

}  // namespace hexl
}  // namespace intel

#endif  // YATFHE_ORACLE_HEXL_SHIM_HPP
