// diffusion_2D_gpu: command-line driver with the flags and the stdout format of the
// reference driver (diffusion_2D/main.cpp, diffusion_2D.cpp UserData/UserOutput), running
// on one GB300 through libstsgpu.so. runtests-diffusion2d.py parses its output unchanged
// (Steps, Error test fails, RHS fn evals, Total simulation time, Maximum relative error).
//
// Problems: --problem periodic (default; the reference code's problem: periodic domain
// [-pi,pi]x[-6,6], Gaussian x sine initial state, optional --inhomogeneous coefficients),
// --problem manufactured (the manufactured-solution Dirichlet benchmark problem on [0,1]^2) or unforced.
// Integrators (main.cpp:236-400): rkc, rkl (LSRKStep STS, fused kernels); erk with a negative
// --order (LSRKStep SSP(2,2), SSP(4,3), SSP(10,4)) or a non-negative one (ARKStep ERK); dirk
// (ARKStep DIRK of --order 2 or 3 with Newton, CG or GMRES and the Jacobi PSetup/PSolve, or
// the PFMG-role multigrid in a hypre build's place when a --pfmg option is given).
#include <algorithm>
#include <chrono>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <iomanip>
#include <iostream>
#include <limits>
#include <sstream>
#include <string>
#include <vector>

#include "stsgpu.h"

using namespace std;

struct Opts {
  // problem (diffusion_2D.hpp:70-93, diffusion_2D.cpp:42-163)
  string problem = "periodic";
  long long nx = 64, ny = 64;
  double kx = 1.0, ky = 1.0, tf = 1.0;
  double xl = -M_PI, xu = M_PI, yl = -6.0, yu = 6.0;
  bool inhomogeneous = false;
  // integrator (main.cpp:24-51)
  string integrator = "rkc";
  double rtol = 1.0e-5, atol = 1.0e-10, hfixed = 0.0, epslin = 0.0;
  int order = 2, controller = 0, maxsteps = 0, onestep = 0, liniters = 20, msbp = 0, smax = 200;
  bool error = false, linear = true, lsinfo = false, prec = true, internaleig = false;
  bool mixed = false, graphs = true;
  string ls = "cg";
  // multigrid preconditioner in hypre PFMG's role (diffusion_2D.cpp:138-150, USE_HYPRE builds)
  bool pfmg = false;
  int pfmg_relax = 2, pfmg_nrelax = 2;
  // output (UserOutput)
  int output = 1, nout = 20;
  // binary checkpoint of the integrator state written at the end / read before the run
  string checkpoint, restart;
};

static bool take(vector<string>& a, const string& key, string* val)
{
  for (size_t i = 0; i < a.size(); ++i)
    if (a[i] == key)
    {
      if (val)
      {
        if (i + 1 >= a.size()) return false;
        *val = a[i + 1];
        a.erase(a.begin() + i, a.begin() + i + 2);
      }
      else a.erase(a.begin() + i);
      return true;
    }
  return false;
}

static void help()
{
  cout << "\nProblem setup command line options:\n"
          "  --problem <periodic|manufactured|unforced>\n"
          "  --nx <nx>  --ny <ny>  --xl --xu --yl --yu  --kx <kx>  --ky <ky>\n"
          "  --inhomogeneous : use spatially-varying diffusion coefficients\n"
          "  --tf <time>     : final time\n"
          "\nIntegrator command line options:\n"
          "  --integrator <dirk|erk|rkc|rkl> --rtol --atol --fixedstep --controller <0..5: PID PI I ExpGus ImpGus ImExGus>\n"
          "  --order <dirk: 2, 3; erk: 2, 3, 4, or -2, -3, -4 for SSP(2,2), SSP(4,3), SSP(10,4)>\n"
          "  --maxsteps --onestep <n> --error --internaleig --smax <stages> --mixed --nographs\n"
          "\nDIRK solver command line options:\n"
          "  --order --nonlinear --ls <cg|gmres> --lsinfo --liniters --epslin --noprec --msbp\n"
          "  --pfmg : CG stage solves preconditioned by the structured multigrid (PFMG role)\n"
          "  --pfmg_relax <type> : 1 = weighted Jacobi, 2 = symmetric, 3 = nonsymmetric red/black Gauss-Seidel\n"
          "  --pfmg_nrelax <num> : pre and post relaxation sweeps\n"
          "\nOutput command line options:\n"
          "  --output <level> (0 = none, 1 = stats, 2 = solution)  --nout <nout>\n"
          "  --checkpoint <file> : write the integrator state at the end of the run\n"
          "  --restart <file>    : continue from a checkpoint written by --checkpoint\n";
}

static int parse(int argc, char** argv, Opts& o)
{
  vector<string> a(argv + 1, argv + argc);
  if (take(a, "--help", nullptr))
  {
    help();
    return 1;
  }
  string v;
  take(a, "--npx", &v); // single GPU: the process grid options are accepted and ignored
  take(a, "--npy", &v);
  if (take(a, "--problem", &v)) o.problem = v;
  if (take(a, "--nx", &v)) o.nx = stoll(v);
  if (take(a, "--ny", &v)) o.ny = stoll(v);
  if (take(a, "--xl", &v)) o.xl = stod(v);
  if (take(a, "--xu", &v)) o.xu = stod(v);
  if (take(a, "--yl", &v)) o.yl = stod(v);
  if (take(a, "--yu", &v)) o.yu = stod(v);
  if (take(a, "--kx", &v)) o.kx = stod(v);
  if (take(a, "--ky", &v)) o.ky = stod(v);
  if (take(a, "--inhomogeneous", nullptr)) o.inhomogeneous = true;
  if (take(a, "--tf", &v)) o.tf = stod(v);
  if (take(a, "--integrator", &v)) o.integrator = v;
  if (take(a, "--rtol", &v)) o.rtol = stod(v);
  if (take(a, "--atol", &v)) o.atol = stod(v);
  if (take(a, "--fixedstep", &v)) o.hfixed = stod(v);
  if (take(a, "--order", &v)) o.order = stoi(v);
  if (take(a, "--controller", &v)) o.controller = stoi(v);
  if (take(a, "--maxsteps", &v)) o.maxsteps = stoi(v);
  if (take(a, "--onestep", &v)) o.onestep = stoi(v);
  if (take(a, "--error", nullptr)) o.error = true;
  if (take(a, "--nonlinear", nullptr)) o.linear = false;
  if (take(a, "--ls", &v)) o.ls = v;
  if (take(a, "--lsinfo", nullptr)) o.lsinfo = true;
  if (take(a, "--liniters", &v)) o.liniters = stoi(v);
  if (take(a, "--msbp", &v)) o.msbp = stoi(v);
  if (take(a, "--epslin", &v)) o.epslin = stod(v);
  if (take(a, "--noprec", nullptr)) o.prec = false;
  if (take(a, "--pfmg", nullptr)) o.pfmg = true;
  if (take(a, "--pfmg_relax", &v))
  {
    o.pfmg_relax = stoi(v);
    o.pfmg       = true;
  }
  if (take(a, "--pfmg_nrelax", &v))
  {
    o.pfmg_nrelax = stoi(v);
    o.pfmg        = true;
  }
  if (take(a, "--internaleig", nullptr)) o.internaleig = true;
  if (take(a, "--smax", &v)) o.smax = stoi(v);
  if (take(a, "--mixed", nullptr)) o.mixed = true;
  if (take(a, "--nographs", nullptr)) o.graphs = false;
  if (take(a, "--output", &v)) o.output = stoi(v);
  if (take(a, "--nout", &v)) o.nout = stoi(v);
  if (take(a, "--checkpoint", &v)) o.checkpoint = v;
  if (take(a, "--restart", &v)) o.restart = v;
  if (!a.empty())
  { // main.cpp:116-132
    cerr << "ERROR: Unknown inputs: ";
    for (auto& s : a) cerr << s << ' ';
    cerr << endl;
    return -1;
  }
  return 0;
}

static int kind_of(const string& p)
{
  if (p == "manufactured") return STS_PROBLEM_MANUFACTURED;
  if (p == "unforced") return STS_PROBLEM_UNFORCED;
  if (p == "periodic") return STS_PROBLEM_PERIODIC;
  return -1;
}

static double urms(N_Vector u, long long nx, long long ny)
{
  return sqrt(N_VDotProd_Sts(u, u) / nx / ny); // diffusion_2D.cpp:801
}

int main(int argc, char** argv)
{
  Opts o;
  int pr = parse(argc, argv, o);
  if (pr > 0) return 0;
  if (pr < 0) return 1;
  const int kind = kind_of(o.problem);
  if (kind < 0)
  {
    cerr << "ERROR: illegal problem" << endl;
    return 1;
  }
  const bool sts  = (o.integrator == "rkc" || o.integrator == "rkl");
  const bool impl = (o.integrator == "dirk");
  const bool expl = (o.integrator == "erk");
  if (!sts && !impl && !expl)
  { // main.cpp:134-139
    cerr << "ERROR: illegal integrator" << endl;
    return 1;
  }
  if (impl && o.ls != "cg" && o.ls != "gmres")
  {
    cerr << "ERROR: illegal linear solver (cg or gmres)" << endl;
    return 1;
  }
  if (impl && o.order != 2 && o.order != 3)
  {
    cerr << "ERROR: dirk orders 2 (ARKODE_SDIRK_2_1_2) and 3 (ARKODE_ARK324L2SA_DIRK_4_2_3)" << endl;
    return 1;
  }
  if (expl && !(o.order == -2 || o.order == -3 || o.order == -4 || (o.order >= 2 && o.order <= 4)))
  { // main.cpp:281-283
    cerr << "ERROR: illegal SSPRK / ERK order (-2, -3, -4 or 2, 3, 4)" << endl;
    return 1;
  }
  if (o.controller < STS_ADAPT_PID || o.controller > STS_ADAPT_IMEX_GUS)
  {
    cerr << "ERROR: illegal controller (0 PID, 1 PI, 2 I, 3 ExpGus, 4 ImpGus, 5 ImExGus)" << endl;
    return 1;
  }
  STS_Context ctx;
  if (STS_ContextCreate(0, &ctx))
  {
    cerr << "ERROR: " << STS_GetLastError() << endl;
    return 1;
  }
  STS_Problem P = STS_ProblemCreate(ctx, kind, o.nx, o.ny, o.kx, o.ky, o.inhomogeneous, o.xl, o.xu, o.yl, o.yu);
  if (!P)
  {
    cerr << "ERROR: " << STS_GetLastError() << endl;
    return 1;
  }
  double dx, dy, cx, cy;
  STS_ProblemGetInfo(P, &dx, &dy, &cx, &cy);
  const long long N = o.nx * o.ny;
  if (o.output > 0)
  { // UserData::print / UserOptions::print / UserOutput::print
    cout << "\n Problem options:\n --------------------------------- \n";
    cout << "  nprocs         = 1\n  kx             = " << o.kx << "\n  ky             = " << o.ky << "\n";
    cout << (o.inhomogeneous ? "  spatially-varying diffusion\n" : "  homogeneous diffusion\n");
    cout << "  tf             = " << o.tf << "\n  nx             = " << o.nx << "\n  ny             = " << o.ny
         << "\n  dx             = " << dx << "\n  dy             = " << dy << "\n";
    cout << " --------------------------------- \n\n Integrator: " << o.integrator << "\n rtol        = " << o.rtol
         << "\n atol        = " << o.atol << "\n controller  = " << o.controller << "\n hfixed      = " << o.hfixed
         << "\n max steps   = " << o.maxsteps << "\n";
    if (sts) cout << (o.internaleig ? " internal eigenvalue estimation\n" : " user-provided dominant eigenvalue\n");
    if (impl && o.pfmg) // diffusion_2D.cpp:217-218
      cout << "  pfmg relaxtype = " << o.pfmg_relax << "\n  pfmg num relax = " << o.pfmg_nrelax << "\n";
    cout << " --------------------------------- \n";
  }
  N_Vector u = N_VNew_Sts(N, ctx);
  STS_Initial(0.0, u, P);
  N_Vector uref = nullptr, uerr = nullptr;
  if (o.error)
  {
    uref = N_VClone_Sts(u);
    uerr = N_VClone_Sts(u);
    N_VScale_Sts(1.0, u, uref);
  }
  void* mem   = nullptr;
  void* ref   = nullptr;
  void* LS    = nullptr; // linear solver of the dirk path (main.cpp:199-231)
  STS_PFMG mg = nullptr; // multigrid preconditioner of the dirk path (--pfmg*)
  if (sts)
  {
    mem = STS_LSRKStepCreateSTS(STS_Diffusion, 0.0, u, ctx);
    STS_LSRKStepSetSTSMethod(mem, o.integrator == "rkc" ? STS_LSRK_RKC_2 : STS_LSRK_RKL_2);
    if (o.internaleig) STS_LSRKStepSetDomEigEstimatorPower(mem, 100, 0.01); // main.cpp:344
    else STS_LSRKStepSetDomEigFn(mem, STS_DomEig);
    STS_LSRKStepSetMaxNumStages(mem, o.smax);
    STS_LSRKStepSetMixedPrecision(mem, o.mixed);
    STS_LSRKStepSetUseGraphs(mem, o.graphs);
  }
  else if (expl && o.order < 0)
  { // main.cpp:250-253, 274-292: SSP methods with 2, 4 and 10 stages
    mem            = STS_LSRKStepCreateSSP(STS_Diffusion, 0.0, u, ctx);
    const int type = o.order == -2 ? STS_LSRK_SSP_S_2 : (o.order == -3 ? STS_LSRK_SSP_S_3 : STS_LSRK_SSP_10_4);
    const int ns   = o.order == -2 ? 2 : (o.order == -3 ? 4 : 10);
    if (STS_LSRKStepSetSSPMethod(mem, type) || STS_LSRKStepSetNumSSPStages(mem, ns))
    {
      cerr << "ERROR: " << STS_GetLastError() << endl;
      return 1;
    }
  }
  else
  { // ARKStep (main.cpp:239-248): explicit ERK or implicit DIRK
    mem = STS_ARKStepCreate(expl ? STS_Diffusion : nullptr, impl ? STS_Diffusion : nullptr, 0.0, u, ctx);
    if (!mem || STS_ARKodeSetOrder(mem, o.order))
    {
      cerr << "ERROR: " << STS_GetLastError() << endl;
      return 1;
    }
  }
  if (impl)
  { // main.cpp:199-231, 300-330
    const int prectype = o.prec ? STS_PREC_RIGHT : STS_PREC_NONE;
    LS = (o.ls == "cg") ? STS_SUNLinSol_PCG(u, prectype, o.liniters, ctx) : STS_SUNLinSol_SPGMR(u, prectype, o.liniters, ctx);
    if (!LS || STS_ARKodeSetLinearSolver(mem, LS, nullptr))
    {
      cerr << "ERROR: " << STS_GetLastError() << endl;
      return 1;
    }
    if (o.prec)
    {
      if (o.pfmg)
      { // the hypre build's PFMG preconditioner (preconditioner_hypre.cpp) in its role
        mg = STS_PFMGCreate(P, o.pfmg_relax, o.pfmg_nrelax);
        if (!mg)
        {
          cerr << "ERROR: " << STS_GetLastError() << endl;
          return 1;
        }
        STS_ARKStepSetPrecData(mem, mg);
        STS_ARKodeSetPreconditioner(mem, STS_PFMGPSetup, STS_PFMGPSolve);
      }
      else STS_ARKodeSetPreconditioner(mem, STS_PSetup, STS_PSolve);
      STS_ARKodeSetLSetupFrequency(mem, o.msbp);
    }
    STS_ARKodeSetEpsLin(mem, o.epslin);
    if (o.linear) STS_ARKodeSetLinear(mem, 0);
  }
  STS_ARKodeSStolerances(mem, o.rtol, o.atol);
  STS_ARKodeSetUserData(mem, P);
  if (o.hfixed > 0.0) STS_ARKodeSetFixedStep(mem, o.hfixed);
  else STS_ARKodeSetAdaptController(mem, o.controller);
  STS_ARKodeSetMaxNumSteps(mem, o.maxsteps > 0 ? o.maxsteps : 500);
  STS_ARKodeSetStopTime(mem, o.tf);
  if (o.error)
  { // main.cpp:387-400: reference integrator (LSRKStep RKC) at rtol 1e-12
    ref = STS_LSRKStepCreateSTS(STS_Diffusion, 0.0, u, ctx);
    STS_ARKodeSStolerances(ref, 1.e-12, o.atol);
    STS_ARKodeSetUserData(ref, P);
    STS_LSRKStepSetDomEigFn(ref, STS_DomEig);
    STS_ARKodeSetMaxNumSteps(ref, 100000LL * (o.maxsteps > 0 ? o.maxsteps : 500));
  }
  int nout      = o.nout;
  int itask     = STS_NORMAL;
  if (o.onestep)
  {
    nout  = o.onestep;
    itask = STS_ONE_STEP;
  }
  double t = 0.0, dTout = o.tf / nout, tout = dTout, errtot = 0.0, simtime = 0.0;
  if (!o.restart.empty())
  {
    if (!sts || STS_LSRKStepReadCheckpoint(mem, o.restart.c_str()) != 0)
    {
      cerr << "ERROR: cannot restart from " << o.restart << ": " << STS_GetLastError() << endl;
      return 1;
    }
    STS_Stats st;
    STS_ARKodeGetStats(mem, &st);
    t = st.t;
    while (tout <= t * (1.0 + 1e-14)) tout += dTout; // the next output time after the checkpoint
    tout = (tout > o.tf) ? o.tf : tout;
    if (o.error && ref)
    { // the self-oracle restarts from the checkpointed state too
      double t2 = 0.0;
      STS_ARKodeSetStopTime(mem, t);
      STS_ARKodeEvolve(mem, t, u, &t2, STS_NORMAL); // copies the restored y_n into u
      STS_ARKodeSetStopTime(mem, o.tf);
      N_VScale_Sts(1.0, u, uref);
      STS_ARKodeReset(ref, t, uref);
    }
  }
  FILE* sol = nullptr;
  cout << scientific << setprecision(numeric_limits<double>::digits10);
  if (o.output > 0)
  {
    cout << "\n          t                     ||u||_rms      \n";
    cout << " ----------------------------------------------\n";
    cout << setw(22) << t << setw(25) << urms(u, o.nx, o.ny) << "\n";
  }
  vector<double> host;
  if (o.output == 2)
  { // UserOutput::open (diffusion_2D.cpp:729-757)
    sol = fopen("diffusion_2d_solution.00000.txt", "w");
    fprintf(sol, "# title Diffusion 2D\n# nvar 1\n# vars u\n# nt  %d\n# nx  %lld\n# xl  %.17g\n# xu  %.17g\n"
                 "# ny  %lld\n# yl  %.17g\n# yu  %.17g\n# px  1\n# py  1\n# np  1\n# is  0\n# ie  %lld\n"
                 "# js  0\n# je  %lld\n",
            nout + 1, o.nx, o.xl, o.xu, o.ny, o.yl, o.yu, o.nx - 1, o.ny - 1);
    host.resize(N);
    N_VCopyToHost_Sts(u, host.data());
    fprintf(sol, "%.15e", t);
    for (double x : host) fprintf(sol, " %.15e", x);
    fprintf(sol, "\n");
  }
  for (int iout = 0; iout < nout; ++iout)
  {
    auto t0 = chrono::steady_clock::now();
    if (o.error) STS_ARKodeSetStopTime(mem, tout); // main.cpp:437-441
    const int flag = STS_ARKodeEvolve(mem, tout, u, &t, itask);
    STS_ContextSynchronize(ctx);
    simtime += chrono::duration<double>(chrono::steady_clock::now() - t0).count();
    if (flag < 0)
    {
      cerr << "\nERROR: ARKodeEvolve returned with flag = " << flag << " (" << STS_GetLastError() << ")\n";
      return 1;
    }
    if (o.error && ref)
    {
      double t2 = 0.0;
      STS_ARKodeSetStopTime(ref, t);
      STS_ARKodeEvolve(ref, t, uref, &t2, STS_NORMAL);
      N_VLinearSum_Sts(1.0, uref, -1.0, u, uerr);
      const double e = N_VMaxNorm_Sts(uerr) / N_VMaxNorm_Sts(uref);
      if (e > errtot) errtot = e;
    }
    if (o.output > 0) cout << setw(22) << t << setw(25) << urms(u, o.nx, o.ny) << "\n";
    if (sol)
    {
      N_VCopyToHost_Sts(u, host.data());
      fprintf(sol, "%.15e", t);
      for (double x : host) fprintf(sol, " %.15e", x);
      fprintf(sol, "\n");
    }
    tout += dTout;
    tout = (tout > o.tf) ? o.tf : tout;
  }
  if (sol) fclose(sol);
  if (!o.checkpoint.empty() && sts && STS_LSRKStepWriteCheckpoint(mem, o.checkpoint.c_str()) != 0)
  {
    cerr << "ERROR: cannot write checkpoint " << o.checkpoint << ": " << STS_GetLastError() << endl;
    return 1;
  }
  if (o.output > 0) cout << " ----------------------------------------------\n\n";
  if (o.error) cout << "Maximum relative error = " << errtot << endl;
  cout << "Total simulation time = " << simtime << endl << endl;
  cout << "Final integrator statistics:" << endl;
  {
    char buf[4096];
    STS_ARKodePrintAllStats(mem, buf, sizeof(buf));
    cout << buf;
  }
  if (mg) cout << "Total PFMG iterations        = " << STS_PFMGNumVCycles(mg) << "\n"; // main.cpp:489-492
  if (kind == STS_PROBLEM_MANUFACTURED)
  {
    N_Vector ex = N_VClone_Sts(u);
    STS_Exact(t, ex, P);
    N_VLinearSum_Sts(1.0, u, -1.0, ex, ex);
    N_Vector e2 = N_VClone_Sts(u);
    STS_Exact(t, e2, P);
    cout << "Relative L2 error vs exact    = " << sqrt(N_VDotProd_Sts(ex, ex) / N_VDotProd_Sts(e2, e2)) << "\n";
    N_VDestroy_Sts(ex);
    N_VDestroy_Sts(e2);
  }
  if (mem) STS_ARKodeFree(&mem);
  if (ref) STS_ARKodeFree(&ref);
  if (LS) STS_SUNLinSolFree(LS);
  if (mg) STS_PFMGFree(&mg);
  N_VDestroy_Sts(u);
  if (uref) N_VDestroy_Sts(uref);
  if (uerr) N_VDestroy_Sts(uerr);
  STS_ProblemFree(&P);
  STS_ContextFree(&ctx);
  return 0;
}
