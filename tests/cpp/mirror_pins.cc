// The C++ mirror's host-side restatements, without a GPU:
//   mirror_pins lattice <n>  -> writes sph::GridArrangement(n) (float[3n])
//   mirror_pins speed        -> reads u32 n and float[3n] velocities from
//                               stdin, writes SpeedOf and SpeedNormalized
//                               (float[n] each)
// tests/test_reference_pins.py compares both with the reference's outputs.
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <vector>

#include "sph_fluid_simulation.hpp"

int main(int argc, char** argv) {
  if (argc >= 3 && std::strcmp(argv[1], "lattice") == 0) {
    const auto pos = sph::GridArrangement(static_cast<uint32_t>(std::strtoul(argv[2], nullptr, 10)));
    std::fwrite(pos.data(), sizeof(sph::Vec3), pos.size(), stdout);
    return 0;
  }
  if (argc >= 2 && std::strcmp(argv[1], "speed") == 0) {
    uint32_t n = 0;
    if (std::fread(&n, 4, 1, stdin) != 1) return 2;
    std::vector<sph::Vec3> v(n);
    if (std::fread(v.data(), sizeof(sph::Vec3), n, stdin) != n) return 2;
    std::vector<float> sp(n), nrm(n);
    for (uint32_t i = 0; i < n; ++i) {
      sp[i] = sph::SpeedOf(v[i]);
      nrm[i] = sph::SpeedNormalized(v[i]);
    }
    std::fwrite(sp.data(), 4, n, stdout);
    std::fwrite(nrm.data(), 4, n, stdout);
    return 0;
  }
  return 2;
}
