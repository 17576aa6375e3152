// Compile check: the reference's generic Solve_PCG template, unmodified, driving
// GPU-resident vectors through delfem2::gb300::DeviceVectorView's ADL
// primitives. Built with -fsyntax-only against the reference's headers.
#include <vector>

#include "delfem2/lsitrsol.h"
#include "dfm2g.hpp"

namespace g = delfem2::gb300;

std::vector<double> solve_with_reference_template(g::CMatrixSparse<double> &K, g::CPreconditionerILU<double> &ilu,
                                                  g::DeviceVectorView r, g::DeviceVectorView x,
                                                  g::DeviceVectorView Pr, g::DeviceVectorView p) {
  return delfem2::Solve_PCG(r, x, Pr, p, 1e-10, 1000, K, ilu);
}
