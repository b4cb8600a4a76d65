// Test driver: read_transform_ri (src/POSTHF/motrans.h:12) through the
// drop-in shim.  Reads the MO coefficients from PREFIX.mos (raw doubles),
// calls read_transform_ri(PREFIX, ...) -- which reads PREFIX.rimp2 -- and
// writes Bia to PREFIX.bia.
//
//   shim_ri_file_driver PREFIX nroe nroao naux
#include <cstdlib>
#include <fstream>
#include <iostream>
#include <string>
#include <vector>

#include "../corr_gb300/shim/corr_shim.h"

int main(int argc, char** argv) {
  if (argc != 5) {
    std::cerr << "usage: shim_ri_file_driver PREFIX nroe nroao naux\n";
    return 2;
  }
  const std::string prefix = argv[1];
  const int nroe = std::atoi(argv[2]), nroao = std::atoi(argv[3]), naux = std::atoi(argv[4]);
  const size_t N = nroao, o = nroe / 2;
  std::vector<double> mos(N * N), bia((size_t)naux * o * (N - o));
  std::ifstream f(prefix + ".mos", std::ios::binary);
  if (!f.read(reinterpret_cast<char*>(mos.data()), mos.size() * sizeof(double))) {
    std::cerr << "cannot read " << prefix << ".mos\n";
    return 2;
  }
  read_transform_ri(prefix, nroe, nroao, naux, mos.data(), bia.data());
  std::ofstream g(prefix + ".bia", std::ios::binary);
  g.write(reinterpret_cast<const char*>(bia.data()), bia.size() * sizeof(double));
  return g ? 0 : 1;
}
