// Data layouts shared by the host set-up code and the perturbation kernel.
//
// Perturbation state ordering (n unknowns), chosen so the stage matrix factorises as
// "chains + one 8x8 head block + a rank-2 coupling":
//   0 Φ | 1 δc 2 θc | 3 δb 4 θb 5 F0 6 F1 7 F2 8 G0 9 G1 10 G2 |
//   F3..F_Lγ (photon T tail) | G3..G_Lγ (photon P tail) | N0..N_Lν (massless ν) |
//   ψ_{j,0..Lh} for j = 0..nx-1 (massive ν momentum bins)
// The equations are those of src/models/{gravity,generic_species,photons,neutrinos}.jl and the
// couplings of src/models/cosmologies.jl:85-98.  Every row is written as
//   (J x)_i = cv[sp]·(A x[ip] + C x[inx]) + (cv[dg] + cv[tr])·x[i] + Σ_e cv[e]·x[ecol]
//             + cv[dx]·(x[dxa] - (3k/4) x[dxb]) + cv[phid]·Φ̇(x) + cv[psid]·Ψ(x)
// where cv[] are τ-dependent coefficients and Φ̇(x), Ψ(x) the two metric functionals
// (src/models/gravity.jl:38-39).  The "dx" term keeps the Thomson drag in difference form
// (θ_b - θ_γ), as the reference writes it, so the residual is free of cancellation.
#pragma once
#include <cstdint>

namespace sbz {

constexpr int kMaxNx = 8;       // massive-ν momentum bins
constexpr int kNCV = 48;        // coefficient slots
constexpr int kMaxFun = 16;     // functional terms (Ψ and δρ sums)
constexpr int kMaxExpr = 80;    // coefficient expressions
constexpr int kMaxChains = 12;
// doubles per table node: τ_g, 1/(τ_{g+1}-τ_g), the 14 (value, d/dτ) values, then from kNodePow the
// power-form coefficients a0..a3 of the cubic Hermite interpolant of each of the 7 quantities on
// [τ_g, τ_{g+1}] in s = (τ - τ_g)/(τ_{g+1} - τ_g) (zero on the last node)
constexpr int kNodeStride = 44;
constexpr int kNodePow = 16;

// coefficient slots
enum : int {
  CV_ZERO = 0, CV_ONE, CV_K, CV_KD, CV_TRG, CV_TRN, CV_TRH, CV_THREE, CV_FOUR, CV_K2, CV_4K3, CV_M1,
  CV_MH,       // -ℋ
  CV_M3HCS,    // -3ℋ c_s²
  CV_KDR,      // κ̇ R, R = 4ργ/(3ρb)
  CV_CSK2,     // c_s² k²
  CV_PA,       // -1/(2ℋ)       (Φ̇ = PA·δρ-sum + PB·Φ - ℋ Ψ)
  CV_DRAG_F1,  // -(4/3) κ̇/k
  CV_KD10,     // -κ̇/10
  CV_KD2,      // -κ̇/2
  CV_PB,       // -k²/(3ℋ)
  CV_MASSIVE = 21  // + 3j: k q_j, -dlnf_j, -(k/3) dlnf_j / q_j
};

struct CompDesc {
  double A, C;
  int16_t ip, inx, e0c, e1c, e2c, dxa, dxb, pad;
  uint8_t sp, dg, tr, e0, e1, e2, phid, psid, dx, pad2[7];
};

// base scalars per τ (value and d/dτ), combined by CoefExpr into cv[] and functional weights
enum : int {
  B_ONE = 0, B_K, B_K2, B_IK, B_IK2, B_KD, B_H, B_CS2, B_IA, B_IA2, B_R, B_IH, B_ITAU,
  B_Q = 13,          // + j: q_j = x_j / E_j
  B_IQ = 13 + 8,     // + j: 1/q_j
  B_E = 13 + 16,     // + j: E_j
  B_IE = 13 + 24,    // + j: 1/E_j
  B_COUNT = 13 + 32
};

// value = K1·B[b[0]]·B[b[1]]·B[b[2]] + K2·B[b[3]]·B[b[4]]·B[b[5]]
struct CoefExpr {
  double K1, K2;
  uint8_t b[6];
  int16_t dest;  // < kNCV: cv slot; kNCV + m: Ψ weight m; kNCV + kMaxFun + m: δρ weight m
};

struct ModelDesc {
  int n, Lg, Ln, Lh, nx;
  int oFt, oGt, oN, oH;
  int npsi, nrho;
  int16_t psiComp[kMaxFun], rhoComp[kMaxFun];
  int nchain;
  int16_t chFirst[kMaxChains], chLast[kMaxChains], chAttach[kMaxChains];  // attach: head row or -1
  int nexpr;
};

// per-cosmology constants for the kernels
struct CosmoDesc {
  double tau_start, tau0, taurec;
  double lnt0, idlnt;
  int ntab;
  float lnt0f, idlntf;  // FP32 copies for the table-node guess
  int pad;
  double Oc0, Ob0, Og0, On0, wh, y0, R0, As, ns, kpivot;
  double xq[kMaxNx], Wq[kMaxNx], dlnf[kMaxNx], ixq[kMaxNx];
  CoefExpr expr[kMaxExpr];
};

}  // namespace sbz
