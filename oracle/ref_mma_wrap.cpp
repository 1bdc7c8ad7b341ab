// C entry points over the reference's vendored MMA solver (simplex/ext/mma/MMASolver.cpp,
// dual interior-point MMA), compiled from the reference sources where they lie by
// oracle/ref_build.sh into oracle/_ref/libref_mma.so. TEST INFRASTRUCTURE ONLY: it pins the
// oracle's MMA restatement and generates the committed MMA fixture.
#include "MMASolver.h"

extern "C" {
void* ref_mma_create(int n, int m) { return new MMASolver(n, m); }
void ref_mma_destroy(void* p) { delete static_cast<MMASolver*>(p); }
void ref_mma_update(void* p, double* xval, const double* dfdx, const double* gx, const double* dgdx, const double* xmin,
                    const double* xmax) {
    static_cast<MMASolver*>(p)->Update(xval, dfdx, gx, dgdx, xmin, xmax);
}
}
