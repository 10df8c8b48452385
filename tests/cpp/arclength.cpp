// C++ use of the facade's PathFollowing on the mesh of tests/src/testcantileverbeam.hh (3D): 10x1x1 hexahedra on
// (10, 2, 2), NeoHooke(E = 100, nu = 0.3) + eas<ES>(n), clamped at x = 0, point loads R[y] += lambda at (10,2,2) and
// (10,2,0); PathFollowing(nr, steps, s, ArcLength{}) with NR tol 1e-10, written as a reference user would
// (pathfollowing.hh:185, testpathfollowing.cpp).  argv: eas kind, n_eas, steps, s, expected lambda, expected max |d|.
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <vector>

#include "ikarus_gb300.hpp"

using namespace Ikarus::GB300;

int main(int argc, char** argv) {
  if (argc < 7) return 2;
  const int kind = std::atoi(argv[1]), n_eas = std::atoi(argv[2]), steps = std::atoi(argv[3]);
  const double s = std::atof(argv[4]), want_lambda = std::atof(argv[5]), want_max = std::atof(argv[6]);
  const int nx = 10, ny = 1, nz = 1;
  const double L = 10.0, h = 2.0;
  std::vector<double> X;
  for (int k = 0; k <= nz; ++k)
    for (int j = 0; j <= ny; ++j)
      for (int i = 0; i <= nx; ++i) X.insert(X.end(), {L * i / nx, h * j / ny, h * k / nz});
  std::vector<int32_t> conn;
  for (int ez = 0; ez < nz; ++ez)
    for (int ey = 0; ey < ny; ++ey)
      for (int ex = 0; ex < nx; ++ex)
        for (int v = 0; v < 8; ++v)
          conn.push_back((ex + (v & 1)) + (nx + 1) * ((ey + ((v >> 1) & 1)) + (ny + 1) * (ez + ((v >> 2) & 1))));
  const int nn = (int)X.size() / 3;
  std::vector<uint8_t> fixed(3 * nn, 0);
  int top1 = -1, top2 = -1;
  for (int n = 0; n < nn; ++n) {
    if (std::abs(X[3 * n]) < 1e-8) fixed[3 * n] = fixed[3 * n + 1] = fixed[3 * n + 2] = 1;
    if (X[3 * n] == L && X[3 * n + 1] == h && X[3 * n + 2] == h) top1 = n;
    if (X[3 * n] == L && X[3 * n + 1] == h && X[3 * n + 2] == 0.0) top2 = n;
  }
  try {
    FiniteElements fes(X, conn, toLamesFirstParameterAndShearModulus(100.0, 0.3), static_cast<EAS>(kind), n_eas);
    FERequirements req(fes, 0.0);
    SparseFlatAssembler assembler(fes, fixed);
    assembler.bind(req, DBCOption::Full);
    assembler.bindPointLoads({3 * top1 + 1, 3 * top2 + 1}, {1.0, 1.0});
    LinearSolver ls(SolverTypeTag::gpu_PCG_BlockJacobi);
    NewtonRaphsonConfig cfg;
    cfg.parameters.tol = 1e-10;
    cfg.extended.linear_rtol = 1e-13;
    cfg.extended.linear_rtol_min = 1e-13;
    NewtonRaphson nr(assembler, ls, cfg);
    PathFollowing alc(nr, steps, s, ArcLength{});
    int stepsEnded = 0;
    alc.subscribe([&](ControlMessages m, const ikr_control_state&) {
      if (m == ControlMessages::STEP_ENDED) ++stepsEnded;
    });
    const auto info = alc.run(req);
    const auto d = req.globalSolution();
    double maxDisp = 0;
    for (double v : d) maxDisp = std::max(maxDisp, std::abs(v));
    std::printf("success %d iterations %d maxDisp %.16g lambda %.16g\n", (int)info.success, info.totalIterations,
                maxDisp, req.parameter());
    const bool ok = info.success && std::abs(req.parameter() - want_lambda) <= 1e-9 * std::abs(want_lambda) &&
                    std::abs(maxDisp - want_max) <= 1e-8 * want_max && stepsEnded == steps + 1 &&
                    (int)info.solverInfos.size() == steps + 1;
    return ok ? 0 : 1;
  } catch (const Error& e) {
    std::printf("error: %s\n", e.what());
    return 3;
  }
}
