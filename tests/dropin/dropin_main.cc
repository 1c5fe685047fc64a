// Driver for the drop-in test: the reference's main flow (cpp/main.cc:97-167) with
// the reference's own Hamiltonian and the GB300 headers in place of
// time_evolution_over_terms.hpp and state_vector.hpp.
#include <cmath>
#include <cstdio>

#include "hamiltonian.hpp"
#include "time_evolution_over_terms.hpp"

int main(int argc, char** argv) {
  if (argc < 2) return 2;
  const unsigned P = 7;
  Hamiltonian h = Hamiltonian();
  StateVector sv = h.IngestBroombridge(argv[1], P);
  h.IndexTerms(SpinIndex::HalfUp);
  h.SetTimestep(1.0);
  const unsigned C = nChoosek(h.num_orbitals(), h.num_occupied());
  for (unsigned i = 0; i < C * C; ++i) sv[i] *= 1.0 / std::sqrt((double)(1u << P));
  try {
    time_evolve_over_terms(sv, h, P);
    sv.qift();
    std::vector<double> probs = sv.IdentifyPhaseAmplitudes();
    std::printf("probs[87] = %.6f\n", probs[87]);
    return probs[87] > 0.5 ? 0 : 1;
  } catch (const char* msg) {
    std::printf("error: %s\n", msg);
    return 3;
  }
}
