// A caller written against the C++ surface alone (include/lpg.hpp, which includes lpg.h):
// elliptic_t from a settings file, its Operator on a fixed input, a Krylov solve through
// linearSolver_t with the elliptic's own preconditioner, an ogs_t built from the
// numbering's ids, and Run. Results go to binary files for the test to compare with the
// oracle.
//   surface_test <settings.rc> <out dir>
#include <cmath>
#include <cstdio>
#include <fstream>
#include <sstream>
#include <string>
#include <vector>

#include "lpg.hpp"

using namespace libp;

static void write(const std::string& path, const std::vector<double>& v) {
  std::ofstream f(path, std::ios::binary);
  f.write(reinterpret_cast<const char*>(v.data()), sizeof(double) * v.size());
}

int main(int argc, char** argv) {
  if (argc < 3) {
    std::fprintf(stderr, "usage: surface_test <settings.rc> <out dir>\n");
    return 2;
  }
  std::ifstream in(argv[1]);
  std::stringstream ss;
  ss << in.rdbuf();
  const std::string out = argv[2];
  try {
    settings_t settings;
    settings.parse(ss.str());
    platform_t platform(settings);
    elliptic_t elliptic(platform, settings);
    const dlong N = elliptic.Nglobal;
    comm_t comm;

    // Operator on q[i] = sin(0.37 i)
    std::vector<double> q(N), Aq(N);
    for (dlong i = 0; i < N; ++i) q[i] = std::sin(0.37 * i);
    deviceMemory<dfloat> o_q = platform.malloc<dfloat>(N), o_Aq = platform.malloc<dfloat>(N);
    o_q.copyFrom(q.data(), N);
    elliptic.Operator(o_q, o_Aq);
    o_Aq.copyTo(Aq.data(), N);
    write(out + "/Aq.bin", Aq);

    // linearSolver_t with the solver the settings name, the elliptic's preconditioner
    linearSolver_t ls;
    if (settings.compareSetting("LINEAR SOLVER", "PCG"))
      ls.Setup<LinearSolver::pcg>(N, 0, platform, settings, comm);
    else
      ls.Setup<LinearSolver::fpcg>(N, 0, platform, settings, comm);
    deviceMemory<dfloat> o_r = platform.malloc<dfloat>(N), o_x = platform.malloc<dfloat>(N);
    elliptic.BuildRhs(o_r);
    std::vector<double> x(N, 0.0);
    o_x.copyFrom(x.data(), N);
    const int iters = elliptic.Solve(ls, o_x, o_r, 1e-8, 5000, 0);
    o_x.copyTo(x.data(), N);
    write(out + "/x.bin", x);

    // the same operator wrapped in a user-defined operator_t (2 A) through precon_t/IdentityPrecon
    struct Twice : public operator_t {
      elliptic_t& e;
      explicit Twice(elliptic_t& el) : e(el) {}
      void Operator(deviceMemory<dfloat>& a, deviceMemory<dfloat>& b) override {
        e.Operator(a, b);
        check(lpg_axpy_f64((int64_t)e.Nglobal, 0.0, b.ptr(), 2.0, b.ptr(), nullptr), "Twice");
      }
    } twice(elliptic);
    precon_t ident;
    ident.Setup<IdentityPrecon>(N);
    elliptic.BuildRhs(o_r);
    std::vector<double> x2(N, 0.0);
    o_x.copyFrom(x2.data(), N);
    linearSolver_t cg;
    cg.Setup<LinearSolver::pcg>(N, 0, platform, settings, comm);
    const int itersCG = cg.Solve(twice, ident, o_x, o_r, 1e-10, 20000, 0);
    o_x.copyTo(x2.data(), N);
    write(out + "/x_twice.bin", x2);

    // ogs_t from ids = assembled index + 1 (0 where masked); Gather(Trans) of v[n] = cos(0.11 n)
    memory<dlong> g2l = elliptic.GlobalToLocal();
    const dlong Nl = (dlong)elliptic.Nlocal;
    memory<hlong> ids(Nl);
    for (dlong n = 0; n < Nl; ++n) ids[n] = g2l[n] >= 0 ? (hlong)g2l[n] + 1 : 0;
    ogs::ogs_t ogs;
    ogs.Setup(Nl, ids, comm, ogs::Signed, ogs::Auto, false, false, platform);
    std::vector<double> v(Nl), gv(ogs.Ngather), sv(Nl);
    for (dlong n = 0; n < Nl; ++n) v[n] = std::cos(0.11 * n);
    deviceMemory<dfloat> o_v = platform.malloc<dfloat>(Nl), o_gv = platform.malloc<dfloat>(ogs.Ngather);
    o_v.copyFrom(v.data(), Nl);
    ogs.Gather(o_gv, o_v, 1, ogs::Add, ogs::Trans);
    o_gv.copyTo(gv.data(), ogs.Ngather);
    write(out + "/gather.bin", gv);
    ogs.Scatter(o_v, o_gv, 1, ogs::NoTrans);
    o_v.copyTo(sv.data(), Nl);
    write(out + "/scatter.bin", sv);

    // an error surfaces as libp::exception with the library's status
    int caught = 0;
    try {
      ogs.Gather(o_gv, o_v, 2, ogs::Add, ogs::Trans);
    } catch (const exception& e) {
      caught = (e.status() == LPG_ERR_UNSUPPORTED);
    }

    elliptic_t::RunResult run = elliptic.Run();
    std::printf("{\"Nglobal\": %d, \"Ngather\": %d, \"iterations\": %d, \"iterations_twice\": %d, "
                "\"run_iterations\": %d, \"norm\": %.17g, \"error\": %.17g, \"caught\": %d}\n",
                N, ogs.Ngather, iters, itersCG, run.iterations, run.norm, run.error, caught);
  } catch (const exception& e) {
    std::fprintf(stderr, "libp::exception (%d): %s\n", e.status(), e.what());
    return 1;
  }
  return 0;
}
