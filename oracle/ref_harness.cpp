// Golden-vector harness: drives the UNMODIFIED reference TwoChNRG routines
// (linked from the reference sources by oracle/build_ref.sh) through the
// NRG_main iteration order (src/Main/NRG_main.cpp:282-427) and prints every
// per-iteration quantity at full precision, so that the CPU oracle
// restatement and the GPU path can be pinned against the real reference.
//
// Test infrastructure only: this file never ships in the product.
//
// Usage:
//   ref_harness <model> <Nsites> <Ncutoff> <Lambda> <U> <ed> <Gamma1> <Gamma2|B> [Delta_SC]
//   model: 1chQS   one-channel Anderson, (Q,S) basis   (ModelSwitch SymNo 0 / ModelNo 0)
//          1chQSz  one-channel Anderson, (Q,Sz) basis  (SymNo 2 / ModelNo 0); last arg = B
//          1chQ    one-channel Anderson, (Q) basis     (SymNo 3 / ModelNo 0)
//          1chS    one-channel Anderson with superconducting leads, (S) basis
//                  (SymNo 7 / ModelNo 0)
//          1chSz   the same in the (Sz) basis (SymNo 8 / ModelNo 0); Gamma2|B = B
//   optional 9th argument: Delta_SC of the superconducting leads; optional
//   10th: a chain file ("chi_N e_N" per line) instead of the flat band's
//          2chQS   two-channel Anderson, (Q,S) basis: the impurity H_{-1} of
//                  OneChQS_SetAnderson_Hm1 coupled to both channels through
//                  TwoChQS_HN_MatEl with f_ch1 = f_ch2 = d; last arg = Gamma2
// Output: line records "ITER", "BLK", "EN", "CUT", "THERMO", "OPAVG" (see
// tests/golden/make_golden.py for the parser).
#include <chrono>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <string>
#include <unistd.h>
#include <vector>

#include "NRGclasses.hpp"
#include "NRGfunctions.hpp"
#include "NRGOpMatRules.hpp"
#include "NRG_main.hpp"
#include "TwoChQS.hpp"
#include "NRGbandtypes.hpp"

#ifndef pi
#define pi 3.141592653589793238462643383279502884197169
#endif

int OneChQS_SetSingleSite(CNRGbasisarray& SingleSite);
int OneChQSz_SetSingleSite(CNRGbasisarray& SingleSite);
int TwoChQS_SetSingleSite(CNRGbasisarray* pSingleSite);

static void print_iter(int N, const std::vector<double>& ParamsHN, CNRGarray& Aeig, double Ecut,
                       int nkept) {
  printf("ITER %d", N);
  for (size_t k = 0; k < ParamsHN.size(); ++k) printf(" %.17g", ParamsHN[k]);
  printf("\n");
  printf("BLK %d %d", Aeig.NumBlocks(), Aeig.NQNumbers);
  for (int b = 0; b < Aeig.NumBlocks(); ++b) {
    for (int q = 0; q < Aeig.NQNumbers; ++q) printf(" %.17g", Aeig.GetQNumber(b, q));
    printf(" %d", Aeig.GetBlockSize(b));
  }
  printf("\n");
  printf("EN %d", (int)Aeig.dEn.size());
  for (size_t k = 0; k < Aeig.dEn.size(); ++k) printf(" %.17g", Aeig.dEn[k]);
  printf("\n");
  printf("CUT %.17g %d\n", Ecut, nkept);
}

// Wilson chain of a non-flat hybridization by the reference's Lanczos
// procedure (CNRGchain::SetChainLanczos, NRGchainClass.cpp:234-520), set up as
// CNRGCodeHandler::SetChain does for the band types (NRGcodehandlerClass.cpp:
// 202-400):
//   ref_harness lanczos <kind> <Lambda> <z> <DiscScheme> <BandOffset> <Nsites> [params...]
//   kind: const (params: Gamma0), lorentzian (the six lanc.in values),
//         table (omega, Gamma(omega) pairs, ascending omega)
// Output: "CHAIN n chi_n e_n" lines and "FSQ Fsq".
static int lanczos_main(int argc, char** argv) {
  if (argc < 8) { fprintf(stderr, "usage: lanczos kind Lambda z disc offset Nsites [params]\n"); return 2; }
  std::string kind = argv[2];
  CNRGchain chain(atof(argv[3]));
  chain.z_twist = atof(argv[4]);
  chain.DiscScheme = atoi(argv[5]);
  chain.BandOffset = atof(argv[6]);
  int N = atoi(argv[7]);
  static std::vector<double> prm;
  for (int k = 8; k < argc; ++k) prm.push_back(atof(argv[k]));
  chain.HybFuncParams = &prm;
  if (kind == "const") {
    chain.HybFunction = HybFunc_Const;
    chain.HybFuncWithEn = chain.DiscScheme == 1 ? HybFunc_Const_divEn : HybFunc_Const_timesEn;
  } else if (kind == "lorentzian") {
    chain.HybFunction = HybFunc_Lorentzian;
    chain.HybFuncWithEn = HybFunc_Lorentzian_timesEn;
  } else if (kind == "table") {
    chain.HybFunction = HybFunc_FromFile;
    chain.HybFuncWithEn = chain.DiscScheme == 1 ? HybFunc_FromFile_divEn : HybFunc_FromFile_timesEn;
    if (chain.GetHyb_w(0.0) == 0.0) { chain.HybRef = 1.0; chain.HybRefIsSet = true; }
  } else {
    fprintf(stderr, "unknown band kind %s\n", kind.c_str());
    return 2;
  }
  FILE* real_out = fdopen(dup(fileno(stdout)), "w");
  fflush(stdout);
  dup2(fileno(stderr), fileno(stdout));
  stdout = real_out;
  chain.SetChainLanczos(N);
  for (int n = 0; n < N; ++n) printf("CHAIN %d %.17g %.17g\n", n, chain.GetChin(n), chain.GetEn(n));
  printf("FSQ %.17g\n", chain.Fsq);
  fflush(stdout);
  return 0;
}

int main(int argc, char** argv) {
  if (argc > 1 && std::string(argv[1]) == "lanczos") return lanczos_main(argc, argv);
  if (argc < 9) {
    fprintf(stderr, "usage: %s model Nsites Ncutoff Lambda U ed Gamma1 Gamma2|B\n", argv[0]);
    return 2;
  }
  std::string model = argv[1];
  int Nsites = atoi(argv[2]);
  int Ncutoff = atoi(argv[3]);
  double Lambda = atof(argv[4]);
  double U = atof(argv[5]);
  double ed = atof(argv[6]);
  double Gamma1 = atof(argv[7]);
  double extra = atof(argv[8]);

  // Silence the reference's chatter on stdout: all of it goes to stderr.
  FILE* real_out = fdopen(dup(fileno(stdout)), "w");
  fflush(stdout);
  dup2(fileno(stderr), fileno(stdout));
  stdout = real_out;

  double HalfLambdaFactor = 0.5 * (1.0 + 1.0 / Lambda);  // NRGcodehandlerClass.cpp:142-146, z=1
  CNRGchain chain(Lambda);
  chain.SetChainWilson(Nsites > 100 ? Nsites : 100);      // NRGcodehandlerClass.cpp:222-227
  // optional 10th argument: a file of "chi_N e_N" lines replacing the chain
  // (as CNRGCodeHandler::SetChain would for another band type)
  if (argc > 10) {
    FILE* cf = fopen(argv[10], "r");
    if (!cf) { fprintf(stderr, "cannot read %s\n", argv[10]); return 2; }
    chain.chin.clear(); chain.en.clear();
    double a, b;
    while (fscanf(cf, "%lf %lf", &a, &b) == 2) { chain.chin.push_back(a); chain.en.push_back(b); }
    fclose(cf);
  }
  double ALambda = sqrt(0.5 * log(Lambda) * (Lambda + 1) / (Lambda - 1));  // NRG_main.cpp:205-207

  CNRGarray Aeig;
  CNRGbasisarray AeigCut, Abasis, SingleSite;
  CNRGmatrix HN;
  HN.NeedOld = false;
  HN.UpperTriangular = true;
  HN.CheckForMatEl = Diag_check;
  std::vector<CNRGmatrix> Mats;
  std::vector<int> CommonQNs, totSpos;
  std::vector<double> ParamsHN;
  bool totalS = true;
  int sqnumber = 1;
  int nchan = 1;
  // superconducting leads (1chS, 1chSz): the gap, rescaled every iteration
  double deltaSC = argc > 9 ? atof(argv[9]) : 0.0;

  CNRGmatrix aux;
  if (model == "1chQS") {
    OneChQS_SetSingleSite(SingleSite);
    for (int i = 0; i < 4; ++i) Mats.push_back(aux);
    Mats[0].NeedOld = false; Mats[0].UpperTriangular = false;
    Mats[0].CheckForMatEl = OneChQS_cd_check; Mats[0].CalcMatEl = OneChQS_fN_MatEl;
    CNRGmatrix avg; avg.NeedOld = true; avg.UpperTriangular = false; avg.CalcAvg = true;
    avg.CheckForMatEl = Diag_check; avg.CalcMatEl = ImpOnly_MatEl;
    Mats[1] = avg; Mats[2] = avg; Mats[3] = avg;
    strcpy(Mats[1].MatName, "Ndot"); strcpy(Mats[2].MatName, "NdSq"); strcpy(Mats[3].MatName, "SdSq");
    double chi_m1 = sqrt(2.0 * Gamma1 / pi) / (sqrt(Lambda) * HalfLambdaFactor) * ALambda;
    std::vector<double> P = {Lambda, HalfLambdaFactor, U, ed, chi_m1};
    OneChQS_SetAnderson_Hm1(P, &Aeig, Mats);
    CommonQNs = {2, 0, 1, 0, 1}; totSpos = {1};
    HN.CalcHNMatEl = OneChQS_HN_MatEl;
    ParamsHN = {Lambda, chi_m1, 0.0, 0.0};
  } else if (model == "1chQSz") {
    OneChQSz_SetSingleSite(SingleSite);
    for (int i = 0; i < 4; ++i) Mats.push_back(aux);
    Mats[0].NeedOld = false; Mats[0].CheckForMatEl = OneChQ_cd_check; Mats[0].CalcMatEl = OneChQ_fNup_MatEl;
    Mats[1].NeedOld = false; Mats[1].CheckForMatEl = OneChQ_cd_check; Mats[1].CalcMatEl = OneChQ_fNdn_MatEl;
    CNRGmatrix avg; avg.NeedOld = true; avg.UpperTriangular = false; avg.CalcAvg = true;
    avg.CheckForMatEl = Diag_check; avg.CalcMatEl = ImpOnly_MatEl;
    Mats[2] = avg; Mats[3] = avg;
    strcpy(Mats[2].MatName, "Ndot"); strcpy(Mats[3].MatName, "Szdot");
    std::vector<double> P = {U, ed, Lambda, HalfLambdaFactor, extra};
    OneChQSz_SetAnderson_Hm1(P, &Aeig, Mats);
    CommonQNs = {2, 0, 1, 0, 1}; totSpos.clear();
    HN.CalcHNMatEl = OneChQSz_HN_MatEl;
    double chi_m1 = sqrt(2.0 * Gamma1 / pi) / (sqrt(Lambda) * HalfLambdaFactor) * ALambda;
    ParamsHN = {Lambda, chi_m1, 0.0, 0.0};
    totalS = false;
  } else if (model == "1chQ") {
    // CNRGCodeHandler::SetSingleSite, SymNo 3 (NRGcodehandlerClass.cpp:484-503)
    SingleSite.NQNumbers = 1;
    SingleSite.Nshell = 0;
    SingleSite.QNumbers = {-1.0, 0.0, 1.0};
    SingleSite.BlockBegEnd = {0, 0, 1, 2, 3, 3};
    for (int ii = 0; ii < 4; ++ii) SingleSite.iType.push_back(ii);
    // ModelSwitch SymNo 3, ModelNo 0 (CodeHandler_ModelSwitch.cpp:1138-1200)
    for (int i = 0; i < 4; ++i) Mats.push_back(aux);
    Mats[0].NeedOld = false; Mats[0].CheckForMatEl = OneChQ_cd_check; Mats[0].CalcMatEl = OneChQ_fNup_MatEl;
    Mats[1].NeedOld = false; Mats[1].CheckForMatEl = OneChQ_cd_check; Mats[1].CalcMatEl = OneChQ_fNdn_MatEl;
    CNRGmatrix avg; avg.NeedOld = true; avg.UpperTriangular = false; avg.CalcAvg = true;
    avg.CheckForMatEl = Diag_check; avg.CalcMatEl = ImpOnly_MatEl;
    Mats[2] = avg; Mats[3] = avg;
    strcpy(Mats[2].MatName, "Sz"); strcpy(Mats[3].MatName, "Sz2");
    std::vector<double> P = {U, ed, Lambda, HalfLambdaFactor};
    OneChQ_SetAnderson_Hm1(P, &Aeig, Mats);
    CommonQNs = {1, 0, 0}; totSpos.clear();
    HN.CalcHNMatEl = OneChQ_HN_MatEl;
    double chi_m1 = sqrt(2.0 * Gamma1 / pi) / (sqrt(Lambda) * HalfLambdaFactor) * ALambda;
    ParamsHN = {Lambda, chi_m1, 0.0, 0.0};
    totalS = false;
    sqnumber = -1;  // NRGcodehandlerClass.cpp:762-765
  } else if (model == "1chS") {
    // CNRGCodeHandler::SetSingleSite, SymNo 7 (NRGcodehandlerClass.cpp:538-562)
    SingleSite.NQNumbers = 2;
    SingleSite.Nshell = 0;
    SingleSite.totalS = true;
    SingleSite.Sqnumbers.push_back(0);
    SingleSite.QNumbers = {0.0, 0.0, 0.5, 0.5, 0.5, -0.5};
    SingleSite.BlockBegEnd = {0, 1, 2, 2, 3, 3};
    for (int ii = 0; ii < 4; ++ii) SingleSite.iType.push_back(ii);
    // ModelSwitch SymNo 7, ModelNo 0, calcdens 0 (CodeHandler_ModelSwitch.cpp:1681-1814)
    for (int i = 0; i < 4; ++i) Mats.push_back(aux);
    Mats[0].NeedOld = false; Mats[0].UpperTriangular = false;
    Mats[0].CheckForMatEl = OneChS_cd_check; Mats[0].CalcMatEl = OneChS_fN_MatEl;
    CNRGmatrix avg; avg.NeedOld = true; avg.UpperTriangular = false; avg.CalcAvg = true;
    avg.CheckForMatEl = Diag_check; avg.CalcMatEl = ImpOnly_MatEl;
    Mats[1] = avg; Mats[2] = avg; Mats[3] = avg;
    strcpy(Mats[1].MatName, "Ndot"); strcpy(Mats[2].MatName, "NdSq"); strcpy(Mats[3].MatName, "SdSq");
    std::vector<double> P = {Lambda, HalfLambdaFactor, U, ed};
    OneChS_SetAnderson_Hm1(P, &Aeig, Mats);
    CommonQNs = {1, 0, 0}; totSpos = {0};
    HN.CalcHNMatEl = OneChS_HNsc_MatEl;
    double chi_m1 = sqrt(2.0 * Gamma1 / pi) / (sqrt(Lambda) * HalfLambdaFactor) * ALambda;
    ParamsHN = {Lambda, chi_m1, 0.0, deltaSC};  // e_N, Delta_SC (NRG_main.cpp:264-276)
    totalS = true;
    sqnumber = 0;  // NRGcodehandlerClass.cpp:774-777
  } else if (model == "1chSz") {
    // CNRGCodeHandler::SetSingleSite, SymNo 8 (NRGcodehandlerClass.cpp:564-584)
    SingleSite.NQNumbers = 1;
    SingleSite.Nshell = 0;
    SingleSite.totalS = false;
    SingleSite.QNumbers = {0.0, 0.5, -0.5};
    SingleSite.BlockBegEnd = {0, 1, 2, 2, 3, 3};
    for (int ii = 0; ii < 4; ++ii) SingleSite.iType.push_back(ii);
    // ModelSwitch SymNo 8, ModelNo 0, calcdens 0 (CodeHandler_ModelSwitch.cpp:1825-1970)
    for (int i = 0; i < 5; ++i) Mats.push_back(aux);
    Mats[0].NeedOld = false; Mats[0].UpperTriangular = false;
    Mats[0].CheckForMatEl = OneChSz_cdup_check; Mats[0].CalcMatEl = OneChSz_fNup_MatEl;
    Mats[1].NeedOld = false; Mats[1].UpperTriangular = false;
    Mats[1].CheckForMatEl = OneChSz_cddn_check; Mats[1].CalcMatEl = OneChSz_fNdn_MatEl;
    CNRGmatrix avg; avg.NeedOld = true; avg.UpperTriangular = false; avg.CalcAvg = true;
    avg.CheckForMatEl = Diag_check; avg.CalcMatEl = ImpOnly_MatEl;
    Mats[2] = avg; Mats[3] = avg; Mats[4] = avg;
    strcpy(Mats[2].MatName, "Ndot"); strcpy(Mats[3].MatName, "NdSq"); strcpy(Mats[4].MatName, "SdSq");
    std::vector<double> P = {Lambda, HalfLambdaFactor, U, ed, extra};
    OneChSz_SetAnderson_Hm1(P, &Aeig, Mats);
    CommonQNs = {1, 0, 0}; totSpos.clear();
    HN.CalcHNMatEl = OneChSz_HNsc_MatEl;
    double chi_m1 = sqrt(2.0 * Gamma1 / pi) / (sqrt(Lambda) * HalfLambdaFactor) * ALambda;
    ParamsHN = {Lambda, chi_m1, 0.0, deltaSC};
    totalS = false;
    sqnumber = 0;  // NRGcodehandlerClass.cpp:778-781
  } else if (model == "2chQS") {
    TwoChQS_SetSingleSite(&SingleSite);
    // Impurity H_{-1} and its reduced <||d||> from the one-channel set-up.
    std::vector<CNRGmatrix> M1(4, aux);
    strcpy(M1[1].MatName, "Ndot"); strcpy(M1[2].MatName, "NdSq"); strcpy(M1[3].MatName, "SdSq");
    double chi1 = sqrt(2.0 * Gamma1 / pi) / (sqrt(Lambda) * HalfLambdaFactor) * ALambda;
    double chi2 = sqrt(2.0 * extra / pi) / (sqrt(Lambda) * HalfLambdaFactor) * ALambda;
    std::vector<double> P = {Lambda, HalfLambdaFactor, U, ed, chi1};
    OneChQS_SetAnderson_Hm1(P, &Aeig, M1);
    Mats.push_back(M1[0]);  // f_ch1 = d
    Mats.push_back(M1[0]);  // f_ch2 = d
    Mats.push_back(M1[1]); Mats.push_back(M1[2]); Mats.push_back(M1[3]);
    for (int i = 0; i < 2; ++i) {
      Mats[i].NeedOld = false; Mats[i].UpperTriangular = false;
      Mats[i].CheckForMatEl = TwoChQS_cd_check;
      Mats[i].CalcMatEl = (i == 0) ? TwoChQS_fNch1_MatEl : TwoChQS_fNch2_MatEl;
    }
    for (int i = 2; i < 5; ++i) {
      Mats[i].NeedOld = true; Mats[i].UpperTriangular = false; Mats[i].CalcAvg = true;
      Mats[i].CheckForMatEl = Diag_check; Mats[i].CalcMatEl = ImpOnly_MatEl;
    }
    CommonQNs = {2, 0, 1, 0, 1}; totSpos = {1};
    HN.CalcHNMatEl = TwoChQS_HN_MatEl;
    ParamsHN = {Lambda, chi1, chi2, 0.0, 0.0};
    nchan = 2;
  } else {
    fprintf(stderr, "unknown model %s\n", model.c_str());
    return 2;
  }

  double betabar = 0.727;  // NRG_main.cpp:96
  CutStates(Aeig, AeigCut, Ncutoff);  // NRG_main.cpp:239
  // Op averages for H_{-1} (CalcStuff at NRG_main.cpp:262)
  {
    std::vector<double> Pb = {betabar};
    printf("OPAVG -1");
    for (size_t i = 0; i < Mats.size(); ++i)
      if (Mats[i].CalcAvg) printf(" %s %.17g", Mats[i].MatName, CalcOpAvg(Pb, &AeigCut, &Mats[i], totalS, sqnumber));
    printf("\n");
  }

  ParamsHN[nchan + 1] = chain.GetEn(0);  // NRG_main.cpp:198, 272-273
  for (int N = 0; N < Nsites; ++N) {
    const auto t_iter = std::chrono::steady_clock::now();
    double DN = HalfLambdaFactor * pow(Lambda, (-(N - 1) / 2.0));  // NRG_main.cpp:283
    BuildBasis(CommonQNs, totSpos, &AeigCut, &Abasis, &SingleSite, 0);
    HN.DiagHN(ParamsHN, &Abasis, &SingleSite, &Mats[0], &Aeig, false);
    Aeig.SetKept(Ncutoff);
    int nk = 0;
    for (size_t k = 0; k < Aeig.Kept.size(); ++k) nk += Aeig.Kept[k] ? 1 : 0;
    double Ecut = Aeig.Ecut(Ncutoff);
    print_iter(N, ParamsHN, Aeig, Ecut, nk);
    // Thermodynamics at the four betabar values of CNRGCodeHandler::CalcThermo
    // (NRGcodehandlerClass.cpp:643-672), raw Calc values.
    for (int nc = 1; nc <= 4; ++nc) {
      double bN = betabar * pow(Lambda, (nc - 4) / (2.0 * 4));
      std::vector<double> Pb = {bN};
      printf("THERMO %d %.17g %.17g %.17g %.17g\n", nc, bN, DN / bN,
             CalcSuscep(Pb, &Aeig, sqnumber, totalS), CalcEntropy(Pb, &Aeig, sqnumber, totalS));
    }
    CutStates(Aeig, AeigCut, Ncutoff);
    UpdateMatrices(&SingleSite, &AeigCut, &Abasis, &Mats[0], (int)Mats.size(), false);
    {
      std::vector<double> Pb = {betabar};
      printf("OPAVG %d", N);
      for (size_t i = 0; i < Mats.size(); ++i)
        if (Mats[i].CalcAvg) printf(" %s %.17g", Mats[i].MatName, CalcOpAvg(Pb, &AeigCut, &Mats[i], totalS, sqnumber));
      printf("\n");
    }
    printf("KEPTBLK %d", AeigCut.NumBlocks());
    for (int b = 0; b < AeigCut.NumBlocks(); ++b) printf(" %d", AeigCut.GetBlockSize(b));
    printf("\n");
    // wall seconds of this iteration (the reference routines, one thread)
    printf("TIME %d %.6f\n", N,
           std::chrono::duration<double>(std::chrono::steady_clock::now() - t_iter).count());
    fflush(stdout);
    for (int ich = 0; ich < nchan; ++ich) ParamsHN[ich + 1] = chain.GetChin(N);  // NRG_main.cpp:402-405
    if ((int)ParamsHN.size() > nchan + 2) ParamsHN[nchan + 1] = chain.GetEn(N + 1);  // NRG_main.cpp:408-413
    if (model == "1chS" || model == "1chSz")
      ParamsHN[nchan + 2] = chain.ScaleFactor(N) * deltaSC;  // NRG_main.cpp:414-419
  }
  fflush(stdout);
  return 0;
}
