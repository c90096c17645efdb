// Test-only: a definition for a reference symbol whose real body lives in a
// unit that needs Intel MKL.  It is reachable only from plane fitting, which
// the spatial-statistics path never calls; reaching it is a harness bug.
#include <cstdlib>
#include <iostream>
int eig(t3x3 const&, t3x1&, t3x1&, t3x3&, t3x3&) {
  std::cerr << "ERROR::eig() is not available in the oracle harness" << std::endl;
  std::abort();
}
