// ORACLE — test infrastructure only (see oracle_mesh.cpp header).
// p-multigrid preconditioner restatement (filled in with the pMG rows).
#include "oracle_internal.hpp"

#include <stdexcept>

namespace orc {

struct MG {};

void mg_setup(Elliptic &) { throw std::runtime_error("multigrid not yet restated"); }
void mg_apply(Elliptic &, const double *, double *) { throw std::runtime_error("multigrid not yet restated"); }

} // namespace orc
