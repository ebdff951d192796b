// Host construction of the kernel descriptors (component rows, chains, coefficient expressions).
// The row descriptors encode the perturbation equations of
//   metric/GR                 src/models/gravity.jl:37-42
//   CDM, baryons              src/models/generic_species.jl:46-47, cosmologies.jl:95
//   photons T + P             src/models/photons.jl:28-60
//   massless / massive ν      src/models/neutrinos.jl:22-26, 129-132
// in the generic row form documented in sbz_layout.hpp.
#include "sbz_setup.hpp"
#include <cstring>
#include <cmath>

namespace sbz {

static int Fi(const ModelDesc& M, int l) { return l <= 2 ? 5 + l : M.oFt + l - 3; }
static int Gi(const ModelDesc& M, int l) { return l <= 2 ? 8 + l : M.oGt + l - 3; }
static int Ni(const ModelDesc& M, int l) { return M.oN + l; }
static int Hi(const ModelDesc& M, int j, int l) { return M.oH + j * (M.Lh + 1) + l; }

int build_model(const sbz_model& m, ModelDesc& M, std::vector<CompDesc>& comps) {
  if (m.lmax_gamma < 3 || m.lmax_nu < 3 || m.nx_h < 0 || m.nx_h > kMaxNx || (m.nx_h > 0 && m.lmax_h < 3)) return SBZ_ERR_ARG;
  std::memset(&M, 0, sizeof M);
  M.Lg = m.lmax_gamma; M.Ln = m.lmax_nu; M.Lh = m.nx_h > 0 ? m.lmax_h : 0; M.nx = m.nx_h;
  M.oFt = 11;
  M.oGt = M.oFt + (M.Lg - 2);
  M.oN = M.oGt + (M.Lg - 2);
  M.oH = M.oN + (M.Ln + 1);
  M.n = M.oH + M.nx * (M.Lh + 1);
  const int n = M.n, Z = n;  // index n addresses a zero entry
  comps.assign(n, CompDesc{});
  for (auto& c : comps) {
    c.A = c.C = 0; c.ip = c.inx = c.e0c = c.e1c = c.e2c = c.dxa = c.dxb = (int16_t)Z;
    c.sp = c.dg = c.tr = c.e0 = c.e1 = c.e2 = c.phid = c.psid = c.dx = CV_ZERO;
  }
  auto chain = [&](int i, int ip, int inx, double A, double C, int sp) {
    CompDesc& c = comps[i]; c.ip = (int16_t)ip; c.inx = (int16_t)inx; c.A = A; c.C = C; c.sp = (uint8_t)sp;
  };
  auto hier = [&](auto idx, int L, int sp, int dg, int tr) {  // generic free-streaming hierarchy 0..L
    for (int l = 0; l <= L; ++l) {
      const int i = idx(l);
      if (l < L) chain(i, l > 0 ? idx(l - 1) : Z, idx(l + 1), double(l) / (2 * l + 1), -double(l + 1) / (2 * l + 1), sp);
      else { chain(i, idx(l - 1), Z, 1.0, 0.0, sp); comps[i].tr = (uint8_t)tr; }
      comps[i].dg = (uint8_t)dg;
    }
  };
  // metric and matter
  comps[0].phid = CV_ONE;
  comps[1].e0 = CV_M1; comps[1].e0c = 2; comps[1].phid = CV_THREE;
  comps[2].e0 = CV_MH; comps[2].e0c = 2; comps[2].psid = CV_K2;
  comps[3].e0 = CV_M1; comps[3].e0c = 4; comps[3].e1 = CV_M3HCS; comps[3].e1c = 3; comps[3].phid = CV_THREE;
  comps[4].e0 = CV_MH; comps[4].e0c = 4; comps[4].e1 = CV_CSK2; comps[4].e1c = 3; comps[4].psid = CV_K2;
  comps[4].dx = CV_KDR; comps[4].dxa = 4; comps[4].dxb = (int16_t)Fi(M, 1);
  // photons
  hier([&](int l) { return Fi(M, l); }, M.Lg, CV_K, CV_KD, CV_TRG);
  hier([&](int l) { return Gi(M, l); }, M.Lg, CV_K, CV_KD, CV_TRG);
  comps[Fi(M, 0)].dg = CV_ZERO; comps[Fi(M, 0)].phid = CV_FOUR;
  comps[Fi(M, 1)].dg = CV_ZERO; comps[Fi(M, 1)].psid = CV_4K3;
  comps[Fi(M, 1)].dx = CV_DRAG_F1; comps[Fi(M, 1)].dxa = 4; comps[Fi(M, 1)].dxb = (int16_t)Fi(M, 1);
  for (int r : {Fi(M, 2), Gi(M, 0), Gi(M, 2)}) {
    CompDesc& c = comps[r];
    const int id = (r == Gi(M, 0)) ? CV_KD2 : CV_KD10;
    c.e0 = c.e1 = c.e2 = (uint8_t)id; c.e0c = (int16_t)Fi(M, 2); c.e1c = (int16_t)Gi(M, 0); c.e2c = (int16_t)Gi(M, 2);
  }
  // massless neutrinos
  hier([&](int l) { return Ni(M, l); }, M.Ln, CV_K, CV_ZERO, CV_TRN);
  comps[Ni(M, 0)].phid = CV_FOUR; comps[Ni(M, 1)].psid = CV_4K3;
  // massive neutrinos
  for (int j = 0; j < M.nx; ++j) {
    hier([&](int l) { return Hi(M, j, l); }, M.Lh, CV_MASSIVE + 3 * j, CV_ZERO, CV_TRH);
    comps[Hi(M, j, 0)].phid = (uint8_t)(CV_MASSIVE + 3 * j + 1);
    comps[Hi(M, j, 1)].psid = (uint8_t)(CV_MASSIVE + 3 * j + 2);
  }
  // metric functionals
  M.npsi = 0; M.nrho = 0;
  M.psiComp[M.npsi++] = 0; M.psiComp[M.npsi++] = (int16_t)Fi(M, 2); M.psiComp[M.npsi++] = (int16_t)Ni(M, 2);
  for (int j = 0; j < M.nx; ++j) M.psiComp[M.npsi++] = (int16_t)Hi(M, j, 2);
  M.rhoComp[M.nrho++] = 1; M.rhoComp[M.nrho++] = 3; M.rhoComp[M.nrho++] = (int16_t)Fi(M, 0); M.rhoComp[M.nrho++] = (int16_t)Ni(M, 0);
  for (int j = 0; j < M.nx; ++j) M.rhoComp[M.nrho++] = (int16_t)Hi(M, j, 0);
  // chains for the structured stage solve (eliminated from chLast down to chFirst)
  M.nchain = 0;
  auto addch = [&](int first, int last, int attach) {
    M.chFirst[M.nchain] = (int16_t)first; M.chLast[M.nchain] = (int16_t)last; M.chAttach[M.nchain] = (int16_t)attach; ++M.nchain;
  };
  addch(Fi(M, 3), Fi(M, M.Lg), Fi(M, 2));
  addch(Gi(M, 3), Gi(M, M.Lg), Gi(M, 2));
  addch(Ni(M, 0), Ni(M, M.Ln), -1);
  for (int j = 0; j < M.nx; ++j) addch(Hi(M, j, 0), Hi(M, j, M.Lh), -1);
  M.nexpr = 27 + 5 * M.nx;  // coefficient expressions emitted by build_cosmo
  return SBZ_OK;
}

int build_cosmo(const Background& B, const ModelDesc& M, const sbz_model& m, CosmoDesc& D) {
  std::memset(&D, 0, sizeof D);
  const Cosmo& P = B.P;
  D.tau_start = B.tau_start; D.tau0 = B.tau0; D.taurec = B.taurec;
  D.lnt0 = B.lnt0; D.idlnt = 1.0 / B.dlnt; D.ntab = B.ntab;
  D.lnt0f = (float)D.lnt0; D.idlntf = (float)D.idlnt;
  D.Oc0 = P.Oc0; D.Ob0 = P.Ob0; D.Og0 = P.Og0; D.On0 = P.On0; D.wh = P.wh; D.y0 = P.y0;
  D.R0 = 4.0 / 3.0 * P.Og0 / P.Ob0; D.As = P.As; D.ns = P.ns; D.kpivot = P.kpivot;
  for (int j = 0; j < M.nx; ++j) { D.xq[j] = P.xq[j]; D.Wq[j] = P.Wq[j]; D.dlnf[j] = P.dlnf[j]; D.ixq[j] = 1.0 / P.xq[j]; }
  int ne = 0;
  auto E = [&](int dest, double K1, int a0, int a1 = B_ONE, int a2 = B_ONE, double K2 = 0, int b0 = B_ONE, int b1 = B_ONE, int b2 = B_ONE) {
    CoefExpr& e = D.expr[ne++];
    e.K1 = K1; e.K2 = K2; e.dest = (int16_t)dest;
    e.b[0] = (uint8_t)a0; e.b[1] = (uint8_t)a1; e.b[2] = (uint8_t)a2; e.b[3] = (uint8_t)b0; e.b[4] = (uint8_t)b1; e.b[5] = (uint8_t)b2;
  };
  E(CV_ONE, 1.0, B_ONE);
  E(CV_K, 1.0, B_K);
  E(CV_KD, 1.0, B_KD);
  E(CV_TRG, -(M.Lg + 1.0), B_ITAU);
  E(CV_TRN, -(M.Ln + 1.0), B_ITAU);
  E(CV_TRH, -(M.Lh + 1.0), B_ITAU);
  E(CV_THREE, 3.0, B_ONE);
  E(CV_FOUR, 4.0, B_ONE);
  E(CV_K2, 1.0, B_K2);
  E(CV_4K3, 4.0 / 3.0, B_K);
  E(CV_M1, -1.0, B_ONE);
  E(CV_MH, -1.0, B_H);
  E(CV_M3HCS, -3.0, B_H, B_CS2);
  E(CV_KDR, 1.0, B_KD, B_R);
  E(CV_CSK2, 1.0, B_CS2, B_K2);
  E(CV_PA, -0.5, B_IH);
  E(CV_DRAG_F1, -4.0 / 3.0, B_KD, B_IK);
  E(CV_KD10, -0.1, B_KD);
  E(CV_KD2, -0.5, B_KD);
  E(CV_PB, -1.0 / 3.0, B_K2, B_IH);
  for (int j = 0; j < M.nx; ++j) {
    E(CV_MASSIVE + 3 * j, 1.0, B_K, B_Q + j);
    E(CV_MASSIVE + 3 * j + 1, -P.dlnf[j], B_ONE);
    E(CV_MASSIVE + 3 * j + 2, -P.dlnf[j] / 3.0, B_K, B_IQ + j);
  }
  // Ψ = Φ - (3/k²a²)[Ωγ F2 + Ων N2 + wh Σ W x²/E ψ2]     (src/models/gravity.jl:39)
  const int W0 = kNCV, R0 = kNCV + kMaxFun;
  E(W0 + 0, 1.0, B_ONE);
  E(W0 + 1, -3.0 * P.Og0, B_IA2, B_IK2);
  E(W0 + 2, -3.0 * P.On0, B_IA2, B_IK2);
  for (int j = 0; j < M.nx; ++j) E(W0 + 3 + j, -3.0 * P.wh * P.Wq[j] * P.xq[j] * P.xq[j], B_IA2, B_IK2, B_IE + j);
  // a²δρ·8π/3 = Ωc δc/a + Ωb δb/a + (Ωγ F0 + Ων N0 + wh Σ W E ψ0)/a²   (src/models/gravity.jl:38)
  E(R0 + 0, P.Oc0, B_IA);
  E(R0 + 1, P.Ob0, B_IA);
  E(R0 + 2, P.Og0, B_IA2);
  E(R0 + 3, P.On0, B_IA2);
  for (int j = 0; j < M.nx; ++j) E(R0 + 4 + j, P.wh * P.Wq[j], B_IA2, B_E + j);
  (void)m;
  return ne == M.nexpr ? SBZ_OK : SBZ_ERR_STATE;
}

}  // namespace sbz
