// s4g_solve_case: the standalone C++ driver of libs4g.  It does for a meshed
// OpenFOAM case directory what the OpenFOAM-side solid-model class does
// inside solids4Foam, through the same C ABI and without OpenFOAM:
//   read constant/polyMesh and 0/D            s4g_foam_read_mesh, s4g_foam_read_d
//   load series -> increments                 s4g_foam_load_ramp, s4g_foam_read_time
//   or time steps (other load tables)         s4g_foam_series_kind, s4g_foam_apply_bcs_at,
//                                             s4g_solve_step
//   field relaxation; refuse equation factors s4g_foam_read_relaxation
//   upload the mesh, set law, BCs, controls   s4g_mesh_upload, s4g_material_set,
//                                             s4g_foam_apply_bcs, s4g_solver_set
//   evolve()                                  s4g_solve, s4g_get_gradD
//   after the loop                            s4g_point_interpolate, s4g_derived_fields
// and prints one JSON line with the run's figures.  The model, material and
// controls come from the case (constant/solidProperties,
// constant/mechanicalProperties, system/fvSolution: s4g_foam_read_controls),
// as the reference reads them; command-line options override them.  A total Lagrangian case whose loads are series
// (linear ramps from zero) runs one increment per time step of
// system/controlDict unless --increments is given; a case with other load
// tables (or --time-steps) runs one evolve() per time step, its series
// evaluated at the step's time, as solids4Foam's time loop does.  --plan-only stops after
// the host-side mesh planning and needs no GPU.  --write TIME writes D,
// sigma, sigmaEq and pointD as ASCII fields into <case>/<TIME>/.

#include "s4g.h"

#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <string>
#include <sys/stat.h>
#include <unistd.h>
#include <vector>

namespace {

void usage() {
  std::fprintf(stderr,
               "usage: s4g_solve_case CASE_DIR [options]\n"
               "  (model, law and controls come from the case's constant/solidProperties,\n"
               "   constant/mechanicalProperties and system/fvSolution; options override them)\n"
               "  --model linearGeometryTotalDisplacement | nonLinearGeometryTotalLagrangian |\n"
               "          nonLinearGeometryTotalLagrangianTotalDisplacement\n"
               "  --E E --nu NU            linearElastic (default 200e9, 0.3)\n"
               "  --mu MU --K K            neoHookeanElastic (the total Lagrangian models)\n"
               "  --increments N           load increments of the total Lagrangian models (1)\n"
               "  --time-steps             one evolve() per controlDict time step (the default\n"
               "                           for load tables other than ramps from zero)\n"
               "  --precision FP64|FP32_REFINE\n"
               "  --preconditioner DIC|diagonal  --tolerance T  --relTol R  --maxIter N\n"
               "  --nCorrectors N  --solutionTolerance T  --alternativeTolerance T\n"
               "  --scaleFactor S          RhieChow scale factor (0.1)\n"
               "  --renumber none|RCM|tiled  --part-size N  --dic-subdomains  --ls-full-delta\n"
               "  --device N  --plan-only  --write TIME\n");
}

[[noreturn]] void die(const char* what, s4g_status st) {
  std::fprintf(stderr, "s4g_solve_case: %s: %s (%s)\n", what, s4g_status_str(st), s4g_last_error());
  std::exit(2);
}

void check(s4g_status st, const char* what) {
  if (st != S4G_OK) die(what, st);
}

}  // namespace

int main(int argc, char** argv) {
  if (argc < 2 || !std::strcmp(argv[1], "--help") || !std::strcmp(argv[1], "-h")) {
    usage();
    return argc < 2 ? 1 : 0;
  }
  const std::string caseDir = argv[1];
  std::string modelName, writeTime;
  // the case's own model, law and controls when it has them; else defaults
  s4g_model model = S4G_LIN_GEOM_TOTAL_DISP;
  s4g_law law{};
  law.type = S4G_LINEAR_ELASTIC;
  law.E = 200e9;
  law.nu = 0.3;
  law.mu = 1e6;
  law.K = 2e7;
  s4g_lin_solver lin;
  s4g_outer outer;
  s4g_default_controls(&lin, &outer);
  const bool fromCase = access((caseDir + "/constant/solidProperties").c_str(), R_OK) == 0;
  if (fromCase)
    check(s4g_foam_read_controls(caseDir.c_str(), &model, &law, &lin, &outer),
          "reading the case's solidProperties, mechanicalProperties and fvSolution");
  s4g_mesh_opts mo{S4G_RENUMBER_TILED, 512, 0, 0, 0, 0, nullptr};
  s4g_precision precision = S4G_FP64;
  int increments = 1, device = 0;
  bool planOnly = false, muKGiven = false, eNuGiven = false, incrementsGiven = false;
  bool timeStepsGiven = false;
  bool lsDeltaGiven = false;
  for (int i = 2; i < argc; ++i) {
    const std::string a = argv[i];
    auto val = [&]() -> const char* {
      if (i + 1 >= argc) {
        std::fprintf(stderr, "s4g_solve_case: %s needs a value\n", a.c_str());
        std::exit(1);
      }
      return argv[++i];
    };
    if (a == "--model") modelName = val();
    else if (a == "--E") { law.E = std::atof(val()); eNuGiven = true; }
    else if (a == "--nu") { law.nu = std::atof(val()); eNuGiven = true; }
    else if (a == "--mu") { law.mu = std::atof(val()); muKGiven = true; }
    else if (a == "--K") { law.K = std::atof(val()); muKGiven = true; }
    else if (a == "--increments") { increments = std::atoi(val()); incrementsGiven = true; }
    else if (a == "--time-steps") timeStepsGiven = true;
    else if (a == "--precision") {
      const std::string p = val();
      if (p == "FP64") precision = S4G_FP64;
      else if (p == "FP32_REFINE") precision = S4G_FP32_REFINE;
      else { usage(); return 1; }
    }
    else if (a == "--preconditioner") {
      const std::string p = val();
      if (p == "DIC" || p == "FDIC") lin.preconditioner = S4G_PRECOND_DIC;
      else if (p == "diagonal") lin.preconditioner = S4G_PRECOND_DIAGONAL;
      else { usage(); return 1; }
    }
    else if (a == "--tolerance") lin.tolerance = std::atof(val());
    else if (a == "--relTol") lin.rel_tol = std::atof(val());
    else if (a == "--maxIter") lin.max_iter = std::atoi(val());
    else if (a == "--nCorrectors") outer.n_correctors = std::atoi(val());
    else if (a == "--solutionTolerance") outer.solution_tol = std::atof(val());
    else if (a == "--alternativeTolerance") outer.alternative_tol = std::atof(val());
    else if (a == "--scaleFactor") outer.stab_scale = std::atof(val());
    else if (a == "--renumber") {
      const std::string r = val();
      if (r == "none") mo.renumber = S4G_RENUMBER_NONE;
      else if (r == "RCM") mo.renumber = S4G_RENUMBER_RCM;
      else if (r == "tiled") mo.renumber = S4G_RENUMBER_TILED;
      else { usage(); return 1; }
    }
    else if (a == "--part-size") mo.part_size = std::atoi(val());
    else if (a == "--dic-subdomains") mo.dic_subdomains = 1;
    else if (a == "--ls-full-delta") { mo.ls_boundary_delta = 1; lsDeltaGiven = true; }
    else if (a == "--device") device = std::atoi(val());
    else if (a == "--plan-only") planOnly = true;
    else if (a == "--write") writeTime = val();
    else { usage(); return 1; }
  }
  static const char* const kModels[] = {"linearGeometryTotalDisplacement",
                                        "nonLinearGeometryTotalLagrangian",
                                        "nonLinearGeometryTotalLagrangianTotalDisplacement"};
  if (!modelName.empty()) {
    if (modelName == kModels[0]) model = S4G_LIN_GEOM_TOTAL_DISP;
    else if (modelName == kModels[1]) model = S4G_NONLIN_GEOM_TOTAL_LAG;
    else if (modelName == kModels[2]) model = S4G_NONLIN_GEOM_TOTAL_LAG_TOTAL_DISP;
    else { usage(); return 1; }
  }
  modelName = kModels[(int)model];
  if (muKGiven) law.use_mu_K = 1;
  else if (eNuGiven) law.use_mu_K = 0;
  if (!fromCase && model != S4G_LIN_GEOM_TOTAL_DISP) {
    // no mechanicalProperties: the total Lagrangian models take neoHookeanElastic
    law.type = S4G_NEO_HOOKEAN;
    if (!eNuGiven) law.use_mu_K = 1;
  }

  // the case
  s4g_foam_case* fc = nullptr;
  check(s4g_foam_read_mesh((caseDir + "/constant/polyMesh").c_str(), &fc), "reading constant/polyMesh");
  s4g_mesh_desc desc;
  int nPoints = 0;
  check(s4g_foam_mesh_desc(fc, &desc, &nPoints), "s4g_foam_mesh_desc");
  mo.empty_direction = s4g_foam_empty_direction(fc);  // 2-D: the empty patches' direction
  // the leastSquares boundary delta of the case's gradSchemes (unless given)
  const std::string fvSchemes = caseDir + "/system/fvSchemes";
  if (!lsDeltaGiven && access(fvSchemes.c_str(), R_OK) == 0)
    check(s4g_foam_read_grad_scheme(fvSchemes.c_str(), model == S4G_NONLIN_GEOM_TOTAL_LAG ? "DD" : "D",
                                    &mo.ls_boundary_delta),
          "reading system/fvSchemes");
  s4g_mesh_info info;
  check(s4g_mesh_plan(&desc, &mo, nullptr, &info), "s4g_mesh_plan");
  // the boundary conditions (optional for --plan-only) and their load ramp
  const std::string dFile = caseDir + "/0/D";
  const bool haveD = access(dFile.c_str(), R_OK) == 0;
  if (!planOnly || haveD) check(s4g_foam_read_d(fc, dFile.c_str()), "reading 0/D");
  double rampEnd = 0;
  int constantLoads = 0;
  int seriesKind = 0;
  if (haveD) check(s4g_foam_load_ramp(fc, &rampEnd, &constantLoads), "s4g_foam_load_ramp");
  if (haveD) check(s4g_foam_series_kind(fc, &seriesKind), "s4g_foam_series_kind");
  // time steps: the loads of controlDict's time steps t0 + k dt, k = 1..N
  std::vector<double> stepTimes;
  if (seriesKind == 2 || timeStepsGiven) {
    double t0 = 0, t1 = 0, dt = 0;
    if (s4g_foam_read_time((caseDir + "/system/controlDict").c_str(), &t0, &t1, &dt) != S4G_OK) {
      std::fprintf(stderr, "s4g_solve_case: load tables are stepped through system/controlDict's "
                           "time steps, which cannot be read: %s\n", s4g_last_error());
      return 2;
    }
    const long nSteps = std::max(1L, std::lround((t1 - t0) / dt));
    for (long k = 1; k <= nSteps; ++k) stepTimes.push_back(t0 + (double)k * dt);
    rampEnd = 0;
  }
  if (rampEnd > 0) {
    if (model != S4G_LIN_GEOM_TOTAL_DISP && constantLoads) {
      std::fprintf(stderr, "s4g_solve_case: constant loads beside load series are not built for the "
                           "total Lagrangian models (the increments would ramp them too)\n");
      return 2;
    }
    // The series are applied up to their end value (load factor n/N over the
    // increments), which is the reference's load at endTime only for a run
    // from time 0 to the series' end: any other time window is refused.
    double t0 = 0, t1 = 0, dt = 0;
    if (s4g_foam_read_time((caseDir + "/system/controlDict").c_str(), &t0, &t1, &dt) == S4G_OK) {
      if (t0 != 0.0 || std::fabs(t1 - rampEnd) > 1e-9 * rampEnd) {
        std::fprintf(stderr,
                     "s4g_solve_case: the load series end at %g but the run goes from %g to %g; "
                     "only a run from 0 to the series' end is built\n",
                     rampEnd, t0, t1);
        return 2;
      }
      if (model != S4G_LIN_GEOM_TOTAL_DISP && !incrementsGiven)
        increments = (int)std::lround((t1 - t0) / dt);
    }
  }
  if (increments < 1) {
    std::fprintf(stderr, "s4g_solve_case: increments must be >= 1\n");
    return 1;
  }
  // field relaxation of the solved field is built (s4g_outer.field_relaxation,
  // read with the controls); equation relaxation is not
  const std::string fvSolution = caseDir + "/system/fvSolution";
  if (access(fvSolution.c_str(), R_OK) == 0) {
    const char* solved = model == S4G_NONLIN_GEOM_TOTAL_LAG ? "DD" : "D";
    double fieldFactor = 1, eqnFactor = 1;
    check(s4g_foam_read_relaxation(fvSolution.c_str(), solved, &fieldFactor, &eqnFactor),
          "reading system/fvSolution");
    if (eqnFactor != 1.0) {
      std::fprintf(stderr,
                   "s4g_solve_case: equation relaxationFactors for %s (%g) are not built on the "
                   "GPU path\n",
                   solved, eqnFactor);
      return 2;
    }
    if (!(fieldFactor > 0.0 && fieldFactor <= 1.0)) {
      std::fprintf(stderr, "s4g_solve_case: field relaxation factor %g of %s is not in (0, 1]\n",
                   fieldFactor, solved);
      return 2;
    }
    outer.field_relaxation = fieldFactor;
  }
  if (planOnly) {
    std::printf("{\"case\": \"%s\", \"cells\": %d, \"faces\": %d, \"internal_faces\": %d, "
                "\"points\": %d, \"patches\": %d, \"parts\": %d, \"part_depth\": %d, "
                "\"levels\": %d, \"load_ramp_end\": %g, \"increments\": %d, \"model\": \"%s\", "
                "\"law\": \"%s\", \"E\": %g, \"nu\": %g, \"mu\": %g, \"K\": %g, \"use_mu_K\": %d, "
                "\"nCorrectors\": %d, \"tolerance\": %g, \"relTol\": %g, \"scaleFactor\": %g, "
                "\"empty_direction\": %d, \"fieldRelaxation\": %g, \"ls_boundary_delta\": %d, "
                "\"load_series\": %d, \"time_steps\": %d}\n",
                caseDir.c_str(), desc.n_cells, desc.n_faces, desc.n_internal_faces, nPoints,
                desc.n_patches, info.n_parts, info.part_depth, info.n_levels_global, rampEnd,
                model == S4G_LIN_GEOM_TOTAL_DISP ? 1 : increments, modelName.c_str(),
                law.type == S4G_LINEAR_ELASTIC ? "linearElastic" : "neoHookeanElastic", law.E,
                law.nu, law.mu, law.K, law.use_mu_K, outer.n_correctors, lin.tolerance,
                lin.rel_tol, outer.stab_scale, mo.empty_direction, outer.field_relaxation,
                mo.ls_boundary_delta, seriesKind, (int)stepTimes.size());
    s4g_foam_free(fc);
    return 0;
  }

  // the solve
  s4g_ctx_opts co{device, 0, 0, 0, 0};
  s4g_ctx* ctx = nullptr;
  check(s4g_ctx_create(&ctx, &co), "s4g_ctx_create");
  s4g_mesh* mesh = nullptr;
  check(s4g_mesh_upload(ctx, &desc, &mo, &mesh), "s4g_mesh_upload");
  check(s4g_material_set(mesh, &law), "s4g_material_set");
  check(s4g_foam_apply_bcs(fc, mesh), "applying 0/D");
  check(s4g_solver_set(mesh, &lin, &outer, precision), "s4g_solver_set");
  const int n = desc.n_cells;
  std::vector<double> D(3 * (size_t)n), sigma(6 * (size_t)n), gradD(9 * (size_t)n);
  s4g_perf perf;
  s4g_status st;
  if (stepTimes.empty()) {
    st = s4g_solve(mesh, model, increments, D.data(), sigma.data(), &perf);
    if (st != S4G_OK && st != S4G_NOT_CONVERGED) die("s4g_solve", st);
  } else {
    // solids4Foam's time loop: the boundary conditions at the step's time,
    // then one evolve()
    int corr = 0;
    long long pcg = 0;
    double ms = 0;
    for (double t : stepTimes) {
      check(s4g_foam_apply_bcs_at(fc, mesh, t), "the boundary conditions at a time step");
      st = s4g_solve_step(mesh, model, D.data(), sigma.data(), &perf);
      if (st != S4G_OK && st != S4G_NOT_CONVERGED) die("s4g_solve_step", st);
      if (st == S4G_NOT_CONVERGED)
        std::fprintf(stderr, "time %g: Max iterations reached within momentum loop\n", t);
      corr += perf.n_correctors;
      pcg += perf.total_lin_iters;
      ms += perf.solve_ms;
    }
    perf.n_correctors = corr;
    perf.total_lin_iters = pcg;
    perf.solve_ms = ms;
  }
  if (st == S4G_NOT_CONVERGED) std::fprintf(stderr, "Max iterations reached within momentum loop\n");
  check(s4g_get_gradD(mesh, gradD.data()), "s4g_get_gradD");

  // after the loop
  const double *points = nullptr;
  const int *faceStart = nullptr, *facePoints = nullptr;
  check(s4g_foam_mesh_points(fc, &points, &faceStart, &facePoints), "s4g_foam_mesh_points");
  std::vector<int> pcStart((size_t)nPoints + 1);
  check(s4g_point_cells(nPoints, desc.n_faces, faceStart, facePoints, desc.n_internal_faces,
                        desc.owner, desc.neighbour, pcStart.data(), nullptr), "s4g_point_cells");
  std::vector<int> pcCells((size_t)pcStart[(size_t)nPoints]);
  check(s4g_point_cells(nPoints, desc.n_faces, faceStart, facePoints, desc.n_internal_faces,
                        desc.owner, desc.neighbour, pcStart.data(), pcCells.data()), "s4g_point_cells");
  std::vector<double> pointD(3 * (size_t)nPoints), sigmaEq((size_t)n);
  check(s4g_point_interpolate(nPoints, points, pcStart.data(), pcCells.data(), n, desc.C, D.data(),
                              gradD.data(), pointD.data()), "s4g_point_interpolate");
  check(s4g_derived_fields(n, sigma.data(), gradD.data(), sigmaEq.data(), nullptr, nullptr),
        "s4g_derived_fields");
  double maxD = 0, maxSeq = 0, maxPD = 0;
  for (int c = 0; c < n; ++c) {
    maxD = std::fmax(maxD, std::sqrt(D[3 * c] * D[3 * c] + D[3 * c + 1] * D[3 * c + 1] + D[3 * c + 2] * D[3 * c + 2]));
    maxSeq = std::fmax(maxSeq, sigmaEq[(size_t)c]);
  }
  for (int p = 0; p < nPoints; ++p)
    maxPD = std::fmax(maxPD, std::sqrt(pointD[3 * p] * pointD[3 * p] + pointD[3 * p + 1] * pointD[3 * p + 1] +
                                       pointD[3 * p + 2] * pointD[3 * p + 2]));
  std::printf("{\"case\": \"%s\", \"model\": \"%s\", \"cells\": %d, \"increments\": %d, \"time_steps\": %d, \"status\": \"%s\", "
              "\"converged\": %d, \"correctors\": %d, \"pcg_iterations\": %lld, "
              "\"solve_ms\": %.3f, \"max_mag_D\": %.9g, \"max_mag_pointD\": %.9g, "
              "\"max_sigmaEq\": %.9g}\n",
              caseDir.c_str(), modelName.c_str(), n, model == S4G_LIN_GEOM_TOTAL_DISP ? 1 : increments,
              (int)stepTimes.size(), s4g_status_str(st), perf.converged,
              perf.n_correctors, perf.total_lin_iters, perf.solve_ms, maxD, maxPD, maxSeq);
  if (!writeTime.empty()) {
    // D, sigma, sigmaEq (solidModel::writeFields) and pointD in <case>/<time>
    const std::string tdir = caseDir + "/" + writeTime;
    mkdir(tdir.c_str(), 0755);
    check(s4g_foam_write_point_field(fc, tdir.c_str(), "pointD", "[0 1 0 0 0 0 0]", pointD.data()),
          "writing pointD");
    std::vector<double> Db(3 * (size_t)(desc.n_faces - desc.n_internal_faces));
    check(s4g_foam_boundary_D(fc, D.data(), gradD.data(), Db.data()), "s4g_foam_boundary_D");
    check(s4g_foam_write_field(fc, tdir.c_str(), "D", 3, "[0 1 0 0 0 0 0]", D.data(), Db.data()),
          "writing D");
    check(s4g_foam_write_field(fc, tdir.c_str(), "sigma", 6, "[1 -1 -2 0 0 0 0]", sigma.data(), nullptr),
          "writing sigma");
    check(s4g_foam_write_field(fc, tdir.c_str(), "sigmaEq", 1, "[1 -1 -2 0 0 0 0]", sigmaEq.data(),
                               nullptr),
          "writing sigmaEq");
  }
  s4g_mesh_destroy(mesh);
  s4g_ctx_destroy(ctx);
  s4g_foam_free(fc);
  return st == S4G_OK ? 0 : 3;
}
