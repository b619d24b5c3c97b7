// p-multigrid preconditioner (filled in with the pMG rows).
#include "elliptic.hpp"

namespace nrsg {

struct MGState {};
void MGDeleter::operator()(MGState *m) const { delete m; }

void Elliptic::mg_setup() { throw Error(NRSG_ERR_BAD_CONFIG, "preconditioner = multigrid is not available yet"); }
void Elliptic::mg_apply(const double *, double *) { throw Error(NRSG_ERR_BAD_CONFIG, "multigrid not set up"); }
void Elliptic::mg_release() { mg.reset(); }
std::vector<double> Elliptic::mg_get(const std::string &name)
{
  throw Error(NRSG_ERR_INVALID, "unknown array '" + name + "'");
}

} // namespace nrsg
