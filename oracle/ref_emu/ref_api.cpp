// extern "C" surface over the reference's own solver classes, run on the CUDA stand-in
// (emu.h). TEST INFRASTRUCTURE ONLY: tests/golden/make_ref_golden.py calls it to produce
// the golden vectors that pin the oracle. Vectors are in the reference's blocked solver
// layout; levels count like the reference's (0 = coarsest). The hierarchy is assembled
// as FluidSteadyState3D::init / FluidSteadyState::init assemble it, with the `closed`
// flag given up front (the reference reads it before init_boundary sets it).
#include <cstdint>
#include <cstring>
#include <vector>

#include "DescentSmoother.h"
#include "FluidEnergyGrad.h"
#include "FluidEnergyGrad3D.h"
#include "GMRES.h"
#include "MultigridSolve.h"
#include "StokeFlowDescriptor.h"
#include "StokeFlowDescriptor3D.h"
#include "StokeFlowDirectSolve.h"
#include "StokeFlowMapping.h"
#include "StokeFlowMapping3D.h"
#include "StokeFlowSmoothing.h"
#include "StokeFlowSubSystem.h"
#include "StokeFlowSubSystem3D.h"
#include "StokeLike.h"

// the 2D box smoother's kernel (stoke/StokeFlowSmoothing.cu:74-140), for one colour alone
__global__ void SmoothKernel(Scalar* p, Scalar* vx, Scalar* vy, Scalar* r_p, Scalar* r_vx, Scalar* r_vy, Scalar* area_vx,
                             Scalar* area_vy, Scalar* penalty_p, Scalar* penalty_vx, Scalar* penalty_vy, bool* fixed_p,
                             bool* fixed_vx, bool* fixed_vy, grid2D grid, int flag, Scalar lap_coef);

namespace {

struct DevBuf {
    Scalar* p = nullptr;
    int n = 0;
    void ensure(int m) {
        if (m <= n) return;
        if (p) cudaFree(p);
        cudaMalloc(&p, sizeof(Scalar) * m);
        n = m;
    }
};

struct Ref3 {
    int n = 0, l = 0;
    bool closed = true;
    StokeFlowDescriptor3D* descr = nullptr;  // l levels, finest last
    StokeFlowDescriptor3D energy_descr;
    FluidEnergyGrad3D energy;
    MultigridSolve* mg = nullptr;
    GMRES gmres;
    DevBuf in, out;
};

struct Ref2 {
    int n = 0, l = 0;
    bool closed = true;
    StokeFlowDescriptor* descr = nullptr;
    StokeFlowDescriptor energy_descr;
    FluidEnergyGrad energy;
    MultigridSolve* mg = nullptr;
    StokeFlowDirectSolve* direct = nullptr;
    GMRES gmres;
    DevBuf in, out;
};

template <class F>
void through_device(DevBuf& in, DevBuf& out, int nin, int nout, const double* x, double* y, F f) {
    in.ensure(nin);
    out.ensure(nout);
    cudaMemcpy(in.p, x, sizeof(Scalar) * nin, cudaMemcpyHostToDevice);
    cudaMemset(out.p, 0, sizeof(Scalar) * nout);
    f(out.p, in.p);
    cudaMemcpy(y, out.p, sizeof(Scalar) * nout, cudaMemcpyDeviceToHost);
}

int run_gmres(GMRES& g, LinearMapping* A, const double* b, double* x, int max_iter, double abs_thr, double rel_thr,
              double norm_thr) {
    const int dof = A->xDoF();
    g.max_iter = max_iter;
    g.GMRES_absolute_residual_thres = abs_thr;
    g.GMRES_relative_residual_thres = rel_thr;
    g.GMRES_norm_thres = norm_thr;
    g.verbose = false;
    g.b.resize(dof);
    memcpy(g.b.data(), b, sizeof(Scalar) * dof);
    g.Solve();
    memcpy(x, g.x.data(), sizeof(Scalar) * dof);
    return 0;
}

}  // namespace

extern "C" {

// ---------------------------------------------------------------- 3D
// FluidSteadyState3D::init (stoke/FluidSteadyState3D.cpp:12-90) and FluidEnergy3D::init
// (fluid_topo/FluidEnergy3D.cpp:5-31).
void* ref3_create(int n, int closed) {
    Ref3* h = new Ref3();
    h->n = n;
    h->closed = closed != 0;
    h->l = (int)round(std::log2(n & -n)) - 1;
    const int l = h->l;
    h->descr = new StokeFlowDescriptor3D[l];
    StokeFlowDescriptor3D& d = h->descr[l - 1];
    d.init(n, n, n);
    d.toDevice();
    d.finish();
    h->mg = new MultigridSolve();
    h->mg->init(l);
    for (int i = l - 2; i >= 0; i--) h->descr[i] = createSubSystem(h->descr[i + 1]);
    for (int i = 0; i < l; i++) {
        StokeFlowMapping3DFixed* t0 = new StokeFlowMapping3DFixed();
        t0->init(&h->descr[i]);
        h->mg->mapping[i] = t0;
        if (i != 0) {
            std::vector<LinearMapping*> pred = StokeLike::GenerateJacobiPreconditioner(h->descr[i].grid, t0, 2);
            h->mg->preSmoother[i] = pred[0];
            h->mg->postSmoother[i] = pred[1];
            StokeFlowDownSample3D* t3 = new StokeFlowDownSample3D();
            t3->init(&h->descr[i], &h->descr[i - 1]);
            h->mg->downSample[i - 1] = t3;
            StokeFlowUpSample3D* t4 = new StokeFlowUpSample3D();
            t4->init(&h->descr[i], &h->descr[i - 1]);
            h->mg->upSample[i - 1] = t4;
        } else {
            h->mg->preSmoother[i] = StokeLike::GenerateDirectSolve(h->descr[i].grid, t0, h->closed);
            h->mg->postSmoother[i] = nullptr;
        }
    }
    h->mg->finish();
    h->gmres.linear_mapping = h->mg->mapping[l - 1];
    h->gmres.preconditioner = h->mg;
    h->gmres.Init(50);
    h->gmres.verbose = false;
    h->energy_descr.init(n, n, n);
    h->energy.init(&h->energy_descr);
    return h;
}

int ref3_levels(void* p) { return ((Ref3*)p)->l; }
int ref3_level_dof(void* p, int level) { return ((Ref3*)p)->descr[level].size; }

// init_boundary + update_penalty of FluidSteadyState3D (:92-114, :130-150) and of
// FluidEnergy3D, on finest-level arrays in the blocked layout
void ref3_set_descr(void* p, const double* vol, const uint8_t* fixed, const double* penalty) {
    Ref3* h = (Ref3*)p;
    for (StokeFlowDescriptor3D* d : {&h->descr[h->l - 1], &h->energy_descr}) {
        std::vector<bool> unused;
        bool* fx = new bool[d->size];
        for (int i = 0; i < d->size; i++) fx[i] = fixed[i] != 0;
        d->setFixed(fx);
        d->setVol(const_cast<double*>(vol));
        d->setPenalty(const_cast<double*>(penalty));
        d->toDevice();
        d->finish();
        delete[] fx;
    }
}

// the set-up half of FluidSteadyState3D::solve (:152-156)
void ref3_update(void* p) {
    Ref3* h = (Ref3*)p;
    for (int i = h->l - 2; i >= 0; i--) updateSubSystem(h->descr[i], h->descr[i + 1]);
    h->mg->update();
}
void ref3_update_subsystems(void* p) {
    Ref3* h = (Ref3*)p;
    for (int i = h->l - 2; i >= 0; i--) updateSubSystem(h->descr[i], h->descr[i + 1]);
}
void ref3_level_descr(void* p, int level, double* vol, double* pen, uint8_t* fixed) {
    Ref3* h = (Ref3*)p;
    StokeFlowDescriptor3D& d = h->descr[level];
    std::vector<bool> dummy;
    bool* fx = new bool[d.size];
    cudaMemcpy(vol, d.d_vol, sizeof(Scalar) * d.size, cudaMemcpyDeviceToHost);
    cudaMemcpy(pen, d.d_penalty, sizeof(Scalar) * d.size, cudaMemcpyDeviceToHost);
    cudaMemcpy(fx, d.d_fixed, sizeof(bool) * d.size, cudaMemcpyDeviceToHost);
    for (int i = 0; i < d.size; i++) fixed[i] = fx[i] ? 1 : 0;
    delete[] fx;
}
void ref3_apply_A(void* p, int level, const double* x, double* y) {
    Ref3* h = (Ref3*)p;
    const int s = h->descr[level].size;
    through_device(h->in, h->out, s, s, x, y, [&](Scalar* o, Scalar* i) { h->mg->mapping[level]->applyMapping(o, i); });
}
void ref3_apply_E(void* p, const double* x, double* y) {
    Ref3* h = (Ref3*)p;
    const int s = h->energy_descr.size;
    through_device(h->in, h->out, s, s, x, y, [&](Scalar* o, Scalar* i) { h->energy.applyMapping(o, i); });
}
void ref3_restrict(void* p, int coarse_level, const double* rf, double* rc) {
    Ref3* h = (Ref3*)p;
    through_device(h->in, h->out, h->descr[coarse_level + 1].size, h->descr[coarse_level].size, rf, rc,
                   [&](Scalar* o, Scalar* i) { h->mg->downSample[coarse_level]->applyMapping(o, i); });
}
void ref3_prolong(void* p, int coarse_level, const double* xc, double* xf) {
    Ref3* h = (Ref3*)p;
    through_device(h->in, h->out, h->descr[coarse_level].size, h->descr[coarse_level + 1].size, xc, xf,
                   [&](Scalar* o, Scalar* i) { h->mg->upSample[coarse_level]->applyMapping(o, i); });
}
// one colour's block solve (VelDiagPressureFullSmoothing, stoke/StokeLike.cu:220-278):
// the pre-smoother's first composite member is colour 0, its second colour 1
void ref3_vanka(void* p, int level, int flag, const double* r, double* out) {
    Ref3* h = (Ref3*)p;
    DescentSmoother* ds = static_cast<DescentSmoother*>(h->mg->preSmoother[level]);
    const int s = h->descr[level].size;
    through_device(h->in, h->out, s, s, r, out, [&](Scalar* o, Scalar* i) { ds->P[flag]->applyMapping(o, i); });
}
void ref3_smooth(void* p, int level, int post, const double* r, double* out) {
    Ref3* h = (Ref3*)p;
    LinearMapping* m = post ? h->mg->postSmoother[level] : h->mg->preSmoother[level];
    const int s = h->descr[level].size;
    through_device(h->in, h->out, s, s, r, out, [&](Scalar* o, Scalar* i) { m->applyMapping(o, i); });
}
void ref3_coarse(void* p, const double* r, double* out) {
    Ref3* h = (Ref3*)p;
    const int s = h->descr[0].size;
    through_device(h->in, h->out, s, s, r, out, [&](Scalar* o, Scalar* i) { h->mg->preSmoother[0]->applyMapping(o, i); });
}
void ref3_vcycle(void* p, const double* r, double* out) {
    Ref3* h = (Ref3*)p;
    const int s = h->descr[h->l - 1].size;
    through_device(h->in, h->out, s, s, r, out, [&](Scalar* o, Scalar* i) { h->mg->applyMapping(o, i); });
}
// GMRES::Solve (common_cpx/GMRES.cpp:20-110) with the thresholds given
int ref3_solve(void* p, const double* b, double* x, int max_iter, double abs_thr, double rel_thr, double norm_thr) {
    Ref3* h = (Ref3*)p;
    return run_gmres(h->gmres, h->mg->mapping[h->l - 1], b, x, max_iter, abs_thr, rel_thr, norm_thr);
}

// ---------------------------------------------------------------- 2D
// FluidSteadyState::init (stoke/FluidSteadyState.cpp:9-85) and FluidEnergy::init
// (fluid_topo/FluidEnergy.cpp:5-31).
void* ref2_create(int n, int closed) {
    Ref2* h = new Ref2();
    h->n = n;
    h->closed = closed != 0;
    h->l = (int)round(std::log2(n & -n)) - 2;
    const int l = h->l;
    h->mg = new MultigridSolve();
    h->mg->init(l);
    h->descr = new StokeFlowDescriptor[l];
    StokeFlowDescriptor& d = h->descr[l - 1];
    d.init(n, n);
    d.lap_coeff = (Scalar)1;
    d.toDevice();
    d.finish();
    for (int i = l - 2; i >= 0; i--) h->descr[i] = createSubSystem(h->descr[i + 1]);
    for (int i = 0; i < l; i++) {
        StokeFlowMapping* t0 = new StokeFlowMapping();
        t0->init(&h->descr[i]);
        h->mg->mapping[i] = t0;
        if (i != 0) {
            StokeFlowSmoothing* t1 = new StokeFlowSmoothing();
            t1->init(t0);
            t1->order = 0;
            t1->iter_num = 1;
            h->mg->preSmoother[i] = t1;
            StokeFlowSmoothing* t2 = new StokeFlowSmoothing();
            t2->init(t0);
            t2->order = 1;
            t2->iter_num = 1;
            h->mg->postSmoother[i] = t2;
            StokeFlowDownSample* t3 = new StokeFlowDownSample();
            t3->init(&h->descr[i], &h->descr[i - 1]);
            h->mg->downSample[i - 1] = t3;
            StokeFlowUpSample* t4 = new StokeFlowUpSample();
            t4->init(&h->descr[i], &h->descr[i - 1]);
            h->mg->upSample[i - 1] = t4;
        }
    }
    h->direct = new StokeFlowDirectSolve();
    h->direct->init(&h->descr[0]);
    h->direct->closed = h->closed;
    h->mg->preSmoother[0] = h->direct;
    h->mg->postSmoother[0] = nullptr;
    h->mg->finish();
    h->gmres.linear_mapping = h->mg->mapping[l - 1];
    h->gmres.preconditioner = h->mg;
    h->gmres.Init(40);
    h->gmres.verbose = false;
    h->energy_descr.init(n, n);
    h->energy_descr.toDevice();
    h->energy_descr.finish();
    h->energy.init(&h->energy_descr);
    return h;
}

int ref2_levels(void* p) { return ((Ref2*)p)->l; }
int ref2_level_dof(void* p, int level) { return ((Ref2*)p)->descr[level].size; }

// init_boundary + update_penalty of FluidSteadyState (:87-142) and of FluidEnergy; the
// coarse levels and the coarsest matrix follow the penalty, as there
void ref2_set_descr(void* p, const double* vol, const uint8_t* fixed, const double* penalty) {
    Ref2* h = (Ref2*)p;
    for (StokeFlowDescriptor* d : {&h->descr[h->l - 1], &h->energy_descr}) {
        bool* fx = new bool[d->size];
        for (int i = 0; i < d->size; i++) fx[i] = fixed[i] != 0;
        d->setFixed(fx);
        d->setVol(const_cast<double*>(vol));
        d->setPenalty(const_cast<double*>(penalty));
        d->toDevice();
        d->finish();
        delete[] fx;
    }
    for (int i = h->l - 2; i >= 0; i--) updateSubSystem(h->descr[i], h->descr[i + 1]);
    h->direct->finish();
}
void ref2_level_descr(void* p, int level, double* vol, double* pen, uint8_t* fixed, double* lap) {
    Ref2* h = (Ref2*)p;
    StokeFlowDescriptor& d = h->descr[level];
    bool* fx = new bool[d.size];
    cudaMemcpy(vol, d.d_vol, sizeof(Scalar) * d.size, cudaMemcpyDeviceToHost);
    cudaMemcpy(pen, d.d_penalty, sizeof(Scalar) * d.size, cudaMemcpyDeviceToHost);
    cudaMemcpy(fx, d.d_fixed, sizeof(bool) * d.size, cudaMemcpyDeviceToHost);
    for (int i = 0; i < d.size; i++) fixed[i] = fx[i] ? 1 : 0;
    *lap = d.lap_coeff;
    delete[] fx;
}
void ref2_apply_A(void* p, int level, const double* x, double* y) {
    Ref2* h = (Ref2*)p;
    const int s = h->descr[level].size;
    through_device(h->in, h->out, s, s, x, y, [&](Scalar* o, Scalar* i) { h->mg->mapping[level]->applyMapping(o, i); });
}
void ref2_apply_E(void* p, const double* x, double* y) {
    Ref2* h = (Ref2*)p;
    const int s = h->energy_descr.size;
    through_device(h->in, h->out, s, s, x, y, [&](Scalar* o, Scalar* i) { h->energy.applyMapping(o, i); });
}
void ref2_restrict(void* p, int coarse_level, const double* rf, double* rc) {
    Ref2* h = (Ref2*)p;
    through_device(h->in, h->out, h->descr[coarse_level + 1].size, h->descr[coarse_level].size, rf, rc,
                   [&](Scalar* o, Scalar* i) { h->mg->downSample[coarse_level]->applyMapping(o, i); });
}
void ref2_prolong(void* p, int coarse_level, const double* xc, double* xf) {
    Ref2* h = (Ref2*)p;
    through_device(h->in, h->out, h->descr[coarse_level].size, h->descr[coarse_level + 1].size, xc, xf,
                   [&](Scalar* o, Scalar* i) { h->mg->upSample[coarse_level]->applyMapping(o, i); });
}
// one colour of the box smoother: the kernel launch of StokeFlowSmoothing::applyMapping
// (stoke/StokeFlowSmoothing.cu:190-200) into a zeroed correction
void ref2_smooth_colour(void* p, int level, int flag, const double* r, double* out) {
    Ref2* h = (Ref2*)p;
    StokeFlowDescriptor* d = &h->descr[level];
    const int s = d->size;
    const int c0 = 0, fx0 = d->grid.cell_size(), fy0 = fx0 + d->grid.face_size(0);
    const int Nx = d->Nx, Ny = d->Ny;
    through_device(h->in, h->out, s, s, r, out, [&](Scalar* o, Scalar* i) {
        SmoothKernel<<<dim3(Nx / 8, Ny / 8), dim3(8, 8)>>>(o + c0, o + fx0, o + fy0, i + c0, i + fx0, i + fy0,
                                                           d->d_vol + fx0, d->d_vol + fy0, d->d_penalty + c0,
                                                           d->d_penalty + fx0, d->d_penalty + fy0, d->d_fixed + c0,
                                                           d->d_fixed + fx0, d->d_fixed + fy0, d->grid, flag,
                                                           d->lap_coeff);
    });
}
void ref2_smooth(void* p, int level, int post, const double* r, double* out) {
    Ref2* h = (Ref2*)p;
    LinearMapping* m = post ? h->mg->postSmoother[level] : h->mg->preSmoother[level];
    const int s = h->descr[level].size;
    through_device(h->in, h->out, s, s, r, out, [&](Scalar* o, Scalar* i) { m->applyMapping(o, i); });
}
void ref2_coarse(void* p, const double* r, double* out) {
    Ref2* h = (Ref2*)p;
    const int s = h->descr[0].size;
    through_device(h->in, h->out, s, s, r, out, [&](Scalar* o, Scalar* i) { h->direct->applyMapping(o, i); });
}
void ref2_vcycle(void* p, const double* r, double* out) {
    Ref2* h = (Ref2*)p;
    const int s = h->descr[h->l - 1].size;
    through_device(h->in, h->out, s, s, r, out, [&](Scalar* o, Scalar* i) { h->mg->applyMapping(o, i); });
}
int ref2_solve(void* p, const double* b, double* x, int max_iter, double abs_thr, double rel_thr, double norm_thr) {
    Ref2* h = (Ref2*)p;
    return run_gmres(h->gmres, h->mg->mapping[h->l - 1], b, x, max_iter, abs_thr, rel_thr, norm_thr);
}

}  // extern "C"
