// Registry of the per-class kernel instantiations (host side).
#pragma once
#include "jk_device.cuh"

namespace jk {

constexpr int NPAIRCLASS = (JK_LMAX + 1) * (JK_LMAX + 2) / 2;
constexpr int NQCLASS = NPAIRCLASS * (NPAIRCLASS + 1) / 2;

__host__ __device__ constexpr int pair_class(int li, int lj) { return li * (li + 1) / 2 + lj; }
__host__ __device__ constexpr int pc_li(int pc) { int l = 0; while ((l + 1) * (l + 2) / 2 <= pc) ++l; return l; }
__host__ __device__ constexpr int pc_lj(int pc) { return pc - pc_li(pc) * (pc_li(pc) + 1) / 2; }
__host__ __device__ constexpr int quartet_class(int a, int b) { return a * (a + 1) / 2 + b; }  // a >= b

struct ClassEntry {
    int li, lj, lk, ll;
    int qb64, smem64, qb32, smem32, qbdiag, smemdiag;
    int threads64, threads32;   // block size of the J/K kernels
    int lean64, lean32;         // 1: register-resident kernel, 0: block-cooperative
    const void *k64;     // FP64 J/K kernel
    const void *k32;     // FP32 J/K kernel
    const void *kdiag;   // Schwarz kernel (bra class == ket class only)
    // alternative kernel family for the autotuner (block-cooperative kernel of
    // a class and precision that default to the register-resident one; null
    // otherwise)
    const void *k64_alt;
    const void *k32_alt;
    int smem64_alt, smem32_alt, threads_alt;
    int generic;                // 1: the generic-l kernel (classes with a g shell)
};

// Defined in the instantiation translation units, one per bra pair class.
void register_bra_class_0(ClassEntry *tab);
void register_bra_class_1(ClassEntry *tab);
void register_bra_class_2(ClassEntry *tab);
void register_bra_class_3(ClassEntry *tab);
void register_bra_class_4(ClassEntry *tab);
void register_bra_class_5(ClassEntry *tab);
void register_bra_class_6(ClassEntry *tab);
void register_bra_class_7(ClassEntry *tab);
void register_bra_class_8(ClassEntry *tab);
void register_bra_class_9(ClassEntry *tab);
// classes with a g shell (jk_generic.cu)
void register_generic(ClassEntry *tab);

// ---- nuclear-gradient kernels (jk_grad.cu)

// highest angular momentum of the gradient kernels (the raised 2D integrals
// reach GRAD_LMAX + 1)
#define GRAD_LMAX 3

struct GradDev {
    const double2 *pp_e;      // exponents (a_i, a_j) of every primitive pair
    const int *shell_atom;    // atom of every shell
    const double *dm;         // [n_dm][nao][nao] densities in the sorted Cartesian basis
    int n_dm, nao;
    int qb;                   // quartets (slots) per block of the launch
    double jfac, kfac;        // weights of the J and K density products
    float log_j, log_k;       // their logs plus the density-count factors (screening)
    double *grad;             // [natm][3] accumulators
};

struct GradClass {
    const void *kernel;
    int qb;      // slots per block
    int smem;    // dynamic shared memory of a block
};

// Kernel, slots and shared memory of class (li lj|lk ll); nonzero when a
// shell is above GRAD_LMAX.
int grad_class(int li, int lj, int lk, int ll, GradClass *out);
// Dynamic shared memory limits of the gradient kernels (cudaError_t code).
int grad_set_smem_attrs();

}  // namespace jk
