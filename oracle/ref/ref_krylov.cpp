// The reference's own Krylov templates behind a C ABI, for the oracle tests (test
// infrastructure only: nothing in the package links or loads this).
//
// core/krylov/pamp/pamp/pamp.h (pAMP<cplx>::PropagateVector), core/krylov/gmres/gmres.h
// (GMRES<cplx>::SolveVector) and core/krylov/piram/piram/piram.h (pIRAM<cplx>::Solve) are
// compiled unchanged from the PyProp source tree (oracle/ref/build_ref.py gives the recipe:
// the bundled blitz++ configured out of tree, the shims beside this file for mpi.h,
// boost/shared_ptr.hpp and cblas.h, scipy's bundled BLAS/LAPACK). The operator of each
// method is a caller-supplied callback out = A in on complex128 vectors, as the
// reference's wrappers call back into Python once per product (pampwrapper.cpp:18-46,
// gmreswrapper.cpp, piramsolver.cpp:26-52).
//
// ref_multiply_bandnh restates the generated Fortran kernels
// TensorPotentialMultiply_{Diag,Simp}_BandNH of a rank-2 potential: one BLAS zgbmv per
// angular pair (core/tensorpotential/tensorpotentialmultiply_generator.py:302-432 for the
// pair loops, :622-735 for the zgbmv call), dest += scaling * V * source.
#include <core/krylov/gmres/gmres.h>
#include <core/krylov/pamp/pamp/pamp.h>
#include <core/krylov/piram/piram/piram.h>

#include <exception>
#include <memory>

// core/utility/timer.h declares Start/Stop; the reference defines them over MPI_Wtime
void Timer::Start() { time -= MPI_Wtime(); }
void Timer::Stop() { time += MPI_Wtime(); }

extern "C" {
typedef void (*ref_apply_fn)(void *user, const double *in, double *out, int n);
}

namespace {

class CallbackOperator : public piram::OperatorFunctor<cplx> {
public:
    CallbackOperator(ref_apply_fn fn, void *user) : fn_(fn), user_(user) {}
    void operator()(blitz::Array<cplx, 1> &in, blitz::Array<cplx, 1> &out) override
    {
        if (in.stride(0) != 1 || out.stride(0) != 1) throw std::runtime_error("strided Krylov vector");
        out = 0;  // as the reference's wrappers zero the output before the callback
        fn_(user_, reinterpret_cast<const double *>(in.data()), reinterpret_cast<double *>(out.data()),
            in.extent(0));
    }

private:
    ref_apply_fn fn_;
    void *user_;
};

class StartResidual : public piram::SetupResidualFunctor<cplx> {
public:
    StartResidual(const cplx *v, int n) : v_(v), n_(n) {}
    void operator()(blitz::Array<cplx, 1> &residual) override
    {
        for (int i = 0; i < n_; ++i) residual(i) = v_[i];
    }

private:
    const cplx *v_;
    int n_;
};

blitz::Array<cplx, 1> view(double *p, int n)
{
    return blitz::Array<cplx, 1>(reinterpret_cast<cplx *>(p), blitz::shape(n), blitz::neverDeleteData);
}

}  // namespace

extern "C" {

// ---------------------------------------------------------------------------------- pAMP
struct ref_pamp {
    pamp::pAMP<cplx> p;
};

// exponentiation: 0 Pade (default of the reference), 1 eigenvector decomposition
ref_pamp *ref_pamp_new(int n, int basis_size, int double_ortho, int exponentiation, ref_apply_fn fn, void *user)
{
    try {
        ref_pamp *h = new ref_pamp();
        h->p.MatrixSize = n;
        h->p.BasisSize = basis_size;
        h->p.DisableMPI = true;
        h->p.PerformDoubleOrthogonalization = double_ortho != 0;
        h->p.Exponentiation = (pamp::pAMP<cplx>::ExponentiationMethod)exponentiation;
        h->p.MatrixOperator = piram::OperatorFunctor<cplx>::Ptr(new CallbackOperator(fn, user));
        h->p.Setup();
        return h;
    } catch (const std::exception &) {
        return nullptr;
    }
}

// psi <- exp(-i dt A) psi (complex128, interleaved); err = |last Krylov coefficient|^2
int ref_pamp_propagate(ref_pamp *h, double *psi, double dt_re, double dt_im, double *err, int *ops)
{
    if (!h || !psi) return -1;
    try {
        h->p.ResetStatistics();
        h->p.PropagateVector(view(psi, h->p.MatrixSize), cplx(dt_re, dt_im));
        if (err) *err = h->p.GetPropagationErrorEstimate();
        if (ops) *ops = h->p.GetOperatorCount();
    } catch (const std::exception &) {
        return -2;
    }
    return 0;
}

void ref_pamp_free(ref_pamp *h) { delete h; }

// --------------------------------------------------------------------------------- GMRES
struct ref_gmres {
    gmres::GMRES<cplx> g;
};

ref_gmres *ref_gmres_new(int n, int basis_size, double tolerance, ref_apply_fn fn, void *user)
{
    try {
        ref_gmres *h = new ref_gmres();
        h->g.MatrixSize = n;
        h->g.BasisSize = basis_size;
        h->g.Tolerance = tolerance;
        h->g.DisableMPI = true;
        h->g.MatrixOperator = piram::OperatorFunctor<cplx>::Ptr(new CallbackOperator(fn, user));
        h->g.Setup();
        return h;
    } catch (const std::exception &) {
        return nullptr;
    }
}

// A sol = rhs from sol0 = 0 (the reference's GMRES has no initial guess); err = the final
// least-squares residual estimate, ops = operator applications
int ref_gmres_solve(ref_gmres *h, double *rhs, double *sol, double *err, int *ops)
{
    if (!h || !rhs || !sol) return -1;
    try {
        h->g.ResetStatistics();
        h->g.SolveVector(view(rhs, h->g.MatrixSize), view(sol, h->g.MatrixSize));
        if (err) *err = h->g.GetErrorEstimate();
        if (ops) *ops = h->g.GetOperatorCount();
    } catch (const std::exception &) {
        return -2;
    }
    return 0;
}

void ref_gmres_free(ref_gmres *h) { delete h; }

// --------------------------------------------------------------------------------- pIRAM
// Lowest-real-part eigenpairs (order 0: CompareComplexLessReal, the reference's default;
// 1: CompareComplexGreaterAbs, its inverse-iteration ordering, piramsolver.cpp:79-90).
// start: the initial residual (complex128 [n]); evals: complex [k]; evecs: complex [k][n]
// (may be null); conv: per eigenvalue the convergence estimate (<= 0 converged, [k]).
int ref_piram_solve(int n, int basis_size, int k, double tolerance, int max_restarts, int order,
                    const double *start, ref_apply_fn fn, void *user, double *evals, double *evecs,
                    double *conv, int *restarts, int *ops)
{
    if (n < 1 || k < 1 || 2 * k > basis_size || !start || !evals) return -1;
    try {
        piram::pIRAM<cplx> p;
        p.MatrixSize = n;
        p.BasisSize = basis_size;
        p.EigenvalueCount = k;
        p.Tolerance = tolerance;
        p.MaxRestartCount = max_restarts;
        p.DisableMPI = true;
        p.UseRandomStart = false;
        p.SetupResidual =
            piram::SetupResidualFunctor<cplx>::Ptr(new StartResidual(reinterpret_cast<const cplx *>(start), n));
        p.MatrixOperator = piram::OperatorFunctor<cplx>::Ptr(new CallbackOperator(fn, user));
        if (order == 1) {
            typedef piram::ShiftFunctorSelectRitzValues<cplx, piram::CompareComplexGreaterAbs> shift_t;
            p.CalculateShifts = piram::ShiftFunctor<cplx>::Ptr(new shift_t(piram::CompareComplexGreaterAbs()));
        }
        p.Setup();
        p.Solve();
        p.Postprocess();
        blitz::Array<cplx, 1> ev = p.GetEigenvalues();
        blitz::Array<double, 1> ce = p.GetConvergenceEstimates();
        for (int i = 0; i < k; ++i) {
            evals[2 * i] = ev(i).real();
            evals[2 * i + 1] = ev(i).imag();
            if (conv) conv[i] = ce(i);
            if (evecs) {
                blitz::Array<cplx, 1> v = p.GetEigenvector(i);
                for (int q = 0; q < n; ++q) {
                    evecs[2 * ((size_t)i * n + q)] = v(q).real();
                    evecs[2 * ((size_t)i * n + q) + 1] = v(q).imag();
                }
            }
        }
        if (restarts) *restarts = p.GetRestartCount();
        if (ops) *ops = p.GetOperatorCount();
    } catch (const std::exception &) {
        return -2;
    }
    return 0;
}

// ------------------------------------------------------------------ generated BandNH kernels
// dest[row] += scaling * A_pair * source[col] for every angular pair of a rank-2 potential
// [npairs][N * b] whose radial rank is stored BLAS general-banded (lda = b, (b - 1)/2 sub- and
// super-diagonals): pairs == null is the Diagonal storage (pair p = (p, p)), else the
// Simple storage's [npairs][2] (row, col). One zgbmv per pair, as the generated code.
int ref_multiply_bandnh(const double *potential, int npairs, int N, int b, const int *pairs, double scaling,
                        const double *source, double *dest)
{
    if (!potential || !source || !dest || N < 1 || b < 1 || (b % 2) != 1) return -1;
    const int kb = (b - 1) / 2;
    const cplx alpha(scaling, 0.0), beta(1.0, 0.0);
    const cplx *pot = reinterpret_cast<const cplx *>(potential);
    const cplx *src = reinterpret_cast<const cplx *>(source);
    cplx *dst = reinterpret_cast<cplx *>(dest);
    for (int p = 0; p < npairs; ++p) {
        const int row = pairs ? pairs[2 * p] : p;
        const int col = pairs ? pairs[2 * p + 1] : p;
        cblas_zgbmv(CblasColMajor, CblasNoTrans, N, N, kb, kb, &alpha, pot + (size_t)p * N * b, b,
                    src + (size_t)col * N, 1, &beta, dst + (size_t)row * N, 1);
    }
    return 0;
}

}  // extern "C"
