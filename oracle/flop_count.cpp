// ORACLE — test infrastructure only.  The oracle's beam and contact element
// restatements compiled over flop::Real (flop_real.hpp; with flop_count_beams.cpp
// and flop_count_contact.cpp, which compile the two restatements themselves over
// it, one translation unit each as in the oracle library): reads packed element
// records, evaluates each, and prints the FP64 operations it took.
//
//   flop_count beam    <records.bin> <n> <gauss.bin> <out.bin>
//   flop_count contact <records.bin> <n> <gauss.bin> <out.bin> <surf.bin> <coef.bin> <props.bin>
//
// Records are the oracle's packed input layout (EI_SIZE doubles each); gauss.bin
// holds the weights then the abscissae (3 + 3 doubles), surf.bin the 14-double
// surface record of the oracle's library entry points, props.bin kn, mu, eps_t,
// eta_n.  The element outputs go to out.bin (to check that the counting build
// computes what the oracle computes); one line per record goes to stdout:
// additions/subtractions, multiplications, divisions, square roots, and
// sin/cos/acos calls.
#include <algorithm>
#include <cmath>
#include <cstdint>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <vector>

#include "flop_real.hpp"
#define double flop::Real
#include "eb_oracle.hpp"
#undef double

static std::vector<double> read_all(const char* path) {
  std::vector<double> v;
  FILE* f = std::fopen(path, "rb");
  if (!f) return v;
  double x;
  while (std::fread(&x, sizeof(double), 1, f) == 1) v.push_back(x);
  std::fclose(f);
  return v;
}

int main(int argc, char** argv) {
  if (argc < 6) return 2;
  const bool beam = std::strcmp(argv[1], "beam") == 0;
  const std::vector<double> in = read_all(argv[2]), gq = read_all(argv[4]);
  const int n = std::atoi(argv[3]);
  if ((int64_t)in.size() < (int64_t)n * orc::EI_SIZE || gq.size() < 6) return 3;
  orc::Gauss gs;
  gs.n = 3;
  for (int k = 0; k < 3; ++k) {
    gs.w[k] = flop::Real(gq[k]);
    gs.z[k] = flop::Real(gq[3 + k]);
  }
  const int osz = beam ? orc::EO_SIZE : orc::CO_SIZE;
  std::vector<flop::Real> rec(orc::EI_SIZE), out(osz);
  std::vector<flop::Real> coef;
  orc::Surface srf{};
  orc::ContactProps cp{};
  if (!beam) {
    if (argc < 9) return 2;
    const std::vector<double> s = read_all(argv[6]), c = read_all(argv[7]), p = read_all(argv[8]);
    if (s.size() < 14 || p.size() < 4) return 3;
    coef.assign(c.begin(), c.end());
    srf.kind = (int)s[0];
    srf.axis = srf.kind == 2 ? (int)s[1] : 0;
    srf.position = flop::Real(srf.kind == 2 ? s[2] : 0.0);
    for (int k = 0; k < 3; ++k) srf.center[k] = flop::Real(s[1 + k]);
    srf.radius = flop::Real(s[4]);
    srf.nx = (int64_t)s[5];
    srf.ny = (int64_t)s[6];
    srf.nz = (int64_t)s[7];
    for (int k = 0; k < 3; ++k) {
      srf.x0[k] = flop::Real(s[8 + k]);
      srf.h[k] = flop::Real(s[11 + k]);
    }
    srf.coef = coef.data();
    cp.kn = flop::Real(p[0]);
    cp.mu = flop::Real(p[1]);
    cp.eps_t = flop::Real(p[2]);
    cp.eta_n = flop::Real(p[3]);
  }
  FILE* fo = std::fopen(argv[5], "wb");
  if (!fo) return 4;
  for (int r = 0; r < n; ++r) {
    for (int k = 0; k < orc::EI_SIZE; ++k) rec[k] = flop::Real(in[(int64_t)r * orc::EI_SIZE + k]);
    for (auto& x : out) x = flop::Real(0.0);
    flop::g = flop::Counts{};
    if (beam) orc::compute_beams(rec.data(), gs, out.data());
    else orc::compute_contact_beams(rec.data(), gs, cp, srf, out.data());
    std::printf("%llu %llu %llu %llu %llu\n", flop::g.add, flop::g.mul, flop::g.div, flop::g.sqrt, flop::g.trans);
    for (const auto& x : out) {
      const double v = (double)x;
      std::fwrite(&v, sizeof(double), 1, fo);
    }
  }
  std::fclose(fo);
  return 0;
}
