// Test driver: replays the post-HF part of the reference's main
// (src/main.cc:130-166) through the drop-in shim, with calculate_ri split into
// "integrals from files" + calculate_ri_from_integrals.  Inputs are raw
// little-endian arrays written by tests/test_gpu_shim.py.
//
//   shim_driver DIR nroe nroao naux nrofint
#include <cstdio>
#include <cstdlib>
#include <fstream>
#include <iostream>
#include <string>
#include <vector>

#include "../corr_gb300/shim/corr_shim.h"

template <class T>
static std::vector<T> load(const std::string& path, size_t n) {
  std::vector<T> v(n);
  std::ifstream f(path, std::ios::binary);
  if (!f || !f.read(reinterpret_cast<char*>(v.data()), n * sizeof(T))) {
    std::cerr << "cannot read " << path << '\n';
    std::exit(2);
  }
  return v;
}

int main(int argc, char** argv) {
  if (argc != 6) {
    std::cerr << "usage: shim_driver DIR nroe nroao naux nrofint\n";
    return 2;
  }
  const std::string dir = argv[1];
  systeminfo si{};
  si.nroe = std::atoi(argv[2]);
  si.nroao = std::atoi(argv[3]);
  si.naux_2 = std::atoi(argv[4]);
  si.nrofint = std::atoll(argv[5]);
  const size_t N = si.nroao, X = si.naux_2, o = si.nroe / 2;
  auto mos = load<double>(dir + "/mos.bin", N * N);
  auto fmat = load<double>(dir + "/fmat.bin", N * N);
  auto intval = load<double>(dir + "/intval.bin", si.nrofint);
  auto intnums = load<unsigned short>(dir + "/intnums.bin", 4 * si.nrofint);
  auto sc = load<long long>(dir + "/sortcount.bin", 4);
  auto J = load<double>(dir + "/J.bin", X * X);
  auto pmn = load<double>(dir + "/Pmn.bin", X * N * N);

  OEints oe{};
  oe.MOs = mos.data();
  oe.Fmat = fmat.data();
  TEints te{};
  te.intval = intval.data();
  te.intnums = intnums.data();
  for (int k = 0; k < 4; ++k) te.sortcount[k] = sc[k];
  std::cout.precision(17);

  pHF* postHF = new pHF();
  build_FMo(&si, &oe, postHF);                       // main.cc:132
  MOtrans(&si, &oe, &te, postHF);                    // main.cc:136
  run_canonical_mp2(&si, postHF);                    // main.cc:143
  postHF->BPQ = new double[X * N * N];               // main.cc:151
  calculate_ri_from_integrals((int)X, (int)N, J.data(), pmn.data(), postHF->BPQ);
  postHF->Bia = new double[X * o * (N - o)];         // main.cc:160
  transform_ri(&si, &oe, postHF);                    // main.cc:162
  run_canonical_mp2_ri(&si, postHF);                 // main.cc:165
  return 0;
}
