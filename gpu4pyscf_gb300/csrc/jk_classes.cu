// Kernel instantiations for one bra pair class, selected at compile time by
// -DJK_BRA_CLASS=<0..9>; the build compiles this file once per bra class so
// the translation units build in parallel.
#include "jk_kernel.cuh"
#include "jk_lean.cuh"
#include "jk_registry.h"

#ifndef JK_BRA_CLASS
#error "compile with -DJK_BRA_CLASS=<pair class>"
#endif

namespace jk {

// classes whose ERI block plus one root's 2D integrals fit in registers take
// the register-resident kernel: up to 64 values in FP64, and up to 130 in
// FP32, about the same number of 32-bit registers
constexpr int LEAN_MAX = 64;
constexpr int LEAN_MAX_F32 = 130;

template <int LI, int LJ, int LK, int LL>
static void reg_one(ClassEntry *tab) {
    using S64 = ClassShape<LI, LJ, LK, LL, double>;
    using S32 = ClassShape<LI, LJ, LK, LL, float>;
    constexpr int COST = LeanShape<LI, LJ, LK, LL>::COST;
    ClassEntry &e = tab[quartet_class(pair_class(LI, LJ), pair_class(LK, LL))];
    e.li = LI; e.lj = LJ; e.lk = LK; e.ll = LL;
    e.threads_alt = JK_THREADS;
    if constexpr (COST <= LEAN_MAX) {
        e.lean64 = 1;
        e.k64 = (const void *)rys_lean_kernel<LI, LJ, LK, LL, double>;
        e.qb64 = LEAN_THREADS; e.smem64 = LeanSmem<LI, LJ, LK, LL, double>::BYTES; e.threads64 = LEAN_THREADS;
        e.k64_alt = (const void *)rys_class_kernel<LI, LJ, LK, LL, double, MODE_JK>;
        e.smem64_alt = S64::SMEM;
    } else {
        e.lean64 = 0;
        e.k64 = (const void *)rys_class_kernel<LI, LJ, LK, LL, double, MODE_JK>;
        e.qb64 = S64::QB; e.smem64 = S64::SMEM; e.threads64 = JK_THREADS;
        e.k64_alt = nullptr; e.smem64_alt = 0;
    }
    if constexpr (COST <= LEAN_MAX_F32) {
        e.lean32 = 1;
        e.k32 = (const void *)rys_lean_kernel<LI, LJ, LK, LL, float>;
        e.qb32 = LEAN_THREADS; e.smem32 = LeanSmem<LI, LJ, LK, LL, float>::BYTES; e.threads32 = LEAN_THREADS;
        e.k32_alt = (const void *)rys_class_kernel<LI, LJ, LK, LL, float, MODE_JK>;
        e.smem32_alt = S32::SMEM;
    } else {
        e.lean32 = 0;
        e.k32 = (const void *)rys_class_kernel<LI, LJ, LK, LL, float, MODE_JK>;
        e.qb32 = S32::QB; e.smem32 = S32::SMEM; e.threads32 = JK_THREADS;
        e.k32_alt = nullptr; e.smem32_alt = 0;
    }
    if constexpr (LI == LK && LJ == LL) {
        e.kdiag = (const void *)rys_class_kernel<LI, LJ, LK, LL, double, MODE_DIAG>;
        e.qbdiag = S64::QB; e.smemdiag = S64::SMEM;
    } else {
        e.kdiag = nullptr; e.qbdiag = 0; e.smemdiag = 0;
    }
}

template <int A, int B>
static void reg_kets(ClassEntry *tab) {
    reg_one<pc_li(A), pc_lj(A), pc_li(B), pc_lj(B)>(tab);
    if constexpr (B > 0) reg_kets<A, B - 1>(tab);
}

#define JK_CAT2(a, b) a##b
#define JK_CAT(a, b) JK_CAT2(a, b)

void JK_CAT(register_bra_class_, JK_BRA_CLASS)(ClassEntry *tab) {
    reg_kets<JK_BRA_CLASS, JK_BRA_CLASS>(tab);
}

}  // namespace jk
