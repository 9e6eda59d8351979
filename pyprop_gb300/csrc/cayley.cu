// Cayley / Crank-Nicolson step with a device-resident GMRES, captured in a CUDA graph.
//
// Reference: pyprop/propagator/CayleyPropagator.py:71-150 (b = (S - i dt/2 H) psi with H at
// t + |dt|/2, left preconditioner M, GMRES on M^-1 (S + i dt/2 H)) and
// core/krylov/gmres/gmres.h:433-505 (x0 = 0, least squares each iteration, stop when the
// residual estimate is below max(tol, 1e-13) or the basis is full).
//
// Here the whole step is one graph launch: the GMRES iterations form a conditional WHILE
// node whose body ends in a one-thread kernel that applies the Givens rotations to the new
// Hessenberg column, updates the residual estimate and sets the loop condition on the
// device (cudaGraphSetConditional). No host round trip per iteration.
//
// Precision modes:
//   FP64  - the reference scheme in complex128 throughout.
//   mixed - r = b - A psi = -i dt H psi in FP64; a complex64 GMRES (Givens and back
//           substitution in FP32, Gram-Schmidt sums in FP64 across CTAs) solves
//           M^-1 A d = M^-1 r to 2e-6 relative; psi += d and r -= A d in FP64; the outer
//           WHILE node repeats while the true residual ||r|| (FP64) is above tol (at most
//           4 passes).
#include "cayley_state.cuh"

#include <algorithm>
#include <cmath>
#include <cstring>

template <typename Rd, typename Rs>
int pg_scale_copy(pg_ctx *ctx, const cx<Rs> *src, cx<Rd> *dst, cx<Rd> *dst2, long long n, const double *inv_scale_dev,
                  double mul);
int pg_axpy(pg_ctx *ctx, cxd a, const cxd *x, cxd *y, long long n);

static const int RING = 64;

// Kernels a step runs, counted on the device as the loops decide (one graph launch hides them):
// FP64 step: scales, matvec, preconditioner solve, norm, init, back-substitution, combine;
//            + matvec, axpy, norm, record when the true residual is requested;
// mixed step: scales, matvec; per refinement pass: convert, preconditioner solve, norm, init,
//            back-substitution, combine, matvec, norm, decide;
// per GMRES iteration: next vector, matvec, preconditioner solve, multidot, 2 GS updates, Givens.
// Each count has one matvec kernel per operator product; an operator with dense radial blocks
// launches one more (pg_op_matvec_kernels).
static const int K_FP64_BASE = 7, K_TRUE_RESID = 4, K_MIXED_BASE = 2, K_MIXED_PASS = 9, K_ITER = 7;
// learned preconditioner (right-preconditioned flexible GMRES): per iteration next vector,
// block solve, features, 3 network products, correction, matvec, multidot, 2 GS updates,
// Givens; per pass convert, norm, init, back-substitution, combine, matvec, norm, decide, commit
static const int K_LEARN_ITER = 12, K_LEARN_PASS = 9;

// ------------------------------------------------------------------------------------
// kernels
// ------------------------------------------------------------------------------------
__global__ void cay_scales_kernel(const StepParams *__restrict__ p, cxd *__restrict__ sc, GmresState *st, int kernels)
{
    const int k = threadIdx.x;
    if (k < PG_MAX_SLOTS) {
        const double hdt = 0.5 * p->dt;
        const cxd h = p->h[k];
        // i*a*h = (-a h.y, a h.x)
        cxd plus, minus, diff;
        if (k == 0) {
            plus = mk<double>(1.0, 0.0);
            minus = mk<double>(1.0, 0.0);
            diff = mk<double>(0.0, 0.0);
        } else {
            plus = mk<double>(-hdt * h.y, hdt * h.x);
            minus = mk<double>(hdt * h.y, -hdt * h.x);
            diff = mk<double>(2.0 * hdt * h.y, -2.0 * hdt * h.x);
        }
        sc[SC_PLUS * PG_MAX_SLOTS + k] = plus;
        sc[SC_MINUS * PG_MAX_SLOTS + k] = minus;
        sc[SC_DIFF * PG_MAX_SLOTS + k] = diff;
        sc[SC_NEGPLUS * PG_MAX_SLOTS + k] = mk<double>(-plus.x, -plus.y);
    }
    if (k == 0) {
        st->stats.iterations = 0;
        st->stats.passes = 0;
        st->stats.true_resid = -1.0;
        st->stats.kernels += kernels;
        st->learned_on = 1;  // each step starts with the learned preconditioner (when configured)
        st->accept = 1;
    }
}

// V[0] = d / ||d||, vcur = V[0]; reset the Givens state; decide whether GMRES runs.
template <typename R>
__global__ void cay_gmres_init_kernel(GmresState *st, const double *__restrict__ nrm, const cx<R> *__restrict__ d,
                                      cx<R> *__restrict__ V0, cx<R> *__restrict__ vcur, long long n, double tol,
                                      double rel_tol, int kernels, cudaGraphConditionalHandle inner,
                                      cudaGraphConditionalHandle outer, int has_outer)
{
    const double b = sqrt(fmax(nrm[0], 0.0));  // nrm: FP64 atomic sum of |d|^2 (cleared by backsolve)
    const double s = b > 0.0 ? 1.0 / b : 0.0;
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x) {
        const cx<R> a = d[i];
        const cx<R> v = mk<R>((R)((double)a.x * s), (R)((double)a.y * s));
        V0[i] = v;
        vcur[i] = v;
    }
    if (blockIdx.x == 0 && threadIdx.x == 0) {
        st->j = 0;
        st->stats.k = 0;
        st->stats.beta0 = b;
        st->stats.resid = b;
        st->beta_last = b;
        st->tol_eff = fmax(tol, rel_tol * b);
        st->g[0] = b;
        st->g[1] = 0.0;
        st->stats.passes += 1;
        st->stats.cum_passes += 1;
        st->stats.kernels += kernels;
        st->cont_inner = b > 0.0 ? 1 : 0;
        if (has_outer >= 0) cudaGraphSetConditional(inner, st->cont_inner ? 1u : 0u);
        (void)outer;
    }
}

// V[j] = w / beta_{j-1} and vcur = V[j] for j > 0 (V[0] comes from the init kernel)
template <typename R>
__global__ void cay_next_vector_kernel(const GmresState *__restrict__ st, cx<R> *__restrict__ V, const cx<R> *__restrict__ w,
                                       cx<R> *__restrict__ vcur, long long n)
{
    const int j = st->j;
    if (j == 0) return;
    const double b = st->beta_last;
    const R s = (R)(b > 0.0 ? 1.0 / b : 0.0);
    cx<R> *Vj = V + (size_t)j * n;
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x) {
        const cx<R> a = w[i];
        const cx<R> v = mk<R>(a.x * s, a.y * s);
        Vj[i] = v;
        vcur[i] = v;
    }
}

// One thread: Hessenberg column j = h1 + h2, subdiagonal ||w||; apply the previous Givens
// rotations, form the new one, update g, store the R column, set the loop condition.
// T is the arithmetic precision of the rotations (float for the complex64 inner solve).
template <typename T>
__global__ void cay_gmres_finalize_kernel(GmresState *st, double *h1, double *h2, double *h3, int m,
                                          cudaGraphConditionalHandle inner,
                                          int use_cond, int kernels)
{
    if (threadIdx.x != 0 || blockIdx.x != 0) return;
    const int j = st->j;
    const int J = j + 1;
    T hx[GM_MAXM + 1], hy[GM_MAXM + 1];
    for (int i = 0; i < J; ++i) {
        hx[i] = (T)(h1[2 * i] + h2[2 * i]);
        hy[i] = (T)(h1[2 * i + 1] + h2[2 * i + 1]);
    }
    const double beta = sqrt(fmax(h3[2 * J], 0.0));
    hx[J] = (T)beta;
    hy[J] = (T)0;
    // the three reductions were FP64 atomic sums: clear them for the next iteration
    for (int i = 0; i < 2 * J + 2; ++i) {
        ((double *)h1)[i] = 0.0;
        ((double *)h2)[i] = 0.0;
        ((double *)h3)[i] = 0.0;
    }
    for (int i = 0; i < j; ++i) {
        const T c = (T)st->cs[i];
        const T sx = (T)st->sn[2 * i], sy = (T)st->sn[2 * i + 1];
        // t = c h_i + s h_{i+1};  h_{i+1} = -conj(s) h_i + c h_{i+1}
        const T tx = c * hx[i] + (sx * hx[i + 1] - sy * hy[i + 1]);
        const T ty = c * hy[i] + (sx * hy[i + 1] + sy * hx[i + 1]);
        const T ux = -(sx * hx[i] + sy * hy[i]) + c * hx[i + 1];
        const T uy = -(sx * hy[i] - sy * hx[i]) + c * hy[i + 1];
        hx[i] = tx; hy[i] = ty;
        hx[i + 1] = ux; hy[i + 1] = uy;
    }
    const T a = hypot(hx[j], hy[j]);
    const T bb = hypot(hx[j + 1], hy[j + 1]);
    const T r = hypot(a, bb);
    T c, sx, sy;
    if (r == (T)0) { c = (T)1; sx = (T)0; sy = (T)0; }
    else if (a == (T)0) { c = (T)0; sx = hx[j + 1] / bb; sy = -hy[j + 1] / bb; }
    else {
        c = a / r;
        // s = (h_j / |h_j|) conj(h_{j+1}) / r
        const T px = hx[j] / a, py = hy[j] / a;
        sx = (px * hx[j + 1] + py * hy[j + 1]) / r;
        sy = (py * hx[j + 1] - px * hy[j + 1]) / r;
    }
    const T rjx = c * hx[j] + (sx * hx[j + 1] - sy * hy[j + 1]);
    const T rjy = c * hy[j] + (sx * hy[j + 1] + sy * hx[j + 1]);
    hx[j] = rjx; hy[j] = rjy;
    st->cs[j] = (double)c;
    st->sn[2 * j] = (double)sx;
    st->sn[2 * j + 1] = (double)sy;
    // g_{j+1} = -conj(s) g_j ; g_j = c g_j
    const T gx = (T)st->g[2 * j], gy = (T)st->g[2 * j + 1];
    const T g1x = -(sx * gx + sy * gy), g1y = -(sx * gy - sy * gx);
    st->g[2 * j] = (double)(c * gx);
    st->g[2 * j + 1] = (double)(c * gy);
    st->g[2 * (j + 1)] = (double)g1x;
    st->g[2 * (j + 1) + 1] = (double)g1y;
    for (int i = 0; i <= j; ++i) {
        st->R[2 * (j * GM_MAXM + i)] = (double)hx[i];
        st->R[2 * (j * GM_MAXM + i) + 1] = (double)hy[i];
    }
    const double resid = (double)hypot(g1x, g1y);
    st->stats.k = J;
    st->stats.resid = resid;
    st->stats.iterations += 1;
    st->stats.cum_iterations += 1;
    st->stats.kernels += kernels;
    st->beta_last = beta;
    const bool bad = !(resid == resid);
    const bool conv = bad || resid <= st->tol_eff || J >= m || !(beta > 1e-300);
    if (!conv) st->j = j + 1;
    st->cont_inner = conv ? 0 : 1;
    if (use_cond) cudaGraphSetConditional(inner, conv ? 0u : 1u);
}

// y = R^-1 g over the k completed columns (one thread, precision T)
template <typename T>
__global__ void cay_backsolve_kernel(GmresState *st, double *nrm)
{
    if (threadIdx.x != 0 || blockIdx.x != 0) return;
    nrm[0] = 0.0;  // the init kernel's atomic norm sum, read by then
    nrm[1] = 0.0;
    const int k = st->stats.k;
    T yx[GM_MAXM], yy[GM_MAXM];
    for (int i = k - 1; i >= 0; --i) {
        T sx = (T)st->g[2 * i], sy = (T)st->g[2 * i + 1];
        for (int q = i + 1; q < k; ++q) {
            const T rx = (T)st->R[2 * (q * GM_MAXM + i)], ry = (T)st->R[2 * (q * GM_MAXM + i) + 1];
            sx -= rx * yx[q] - ry * yy[q];
            sy -= rx * yy[q] + ry * yx[q];
        }
        const T dx = (T)st->R[2 * (i * GM_MAXM + i)], dy = (T)st->R[2 * (i * GM_MAXM + i) + 1];
        const T den = dx * dx + dy * dy;
        if (den > (T)0) {
            yx[i] = (sx * dx + sy * dy) / den;
            yy[i] = (sy * dx - sx * dy) / den;
        } else {
            yx[i] = (T)0;
            yy[i] = (T)0;
        }
    }
    for (int i = 0; i < k; ++i) {
        st->y[2 * i] = (double)yx[i];
        st->y[2 * i + 1] = (double)yy[i];
    }
}

// out = V y over k = st->stats.k vectors (complex128 result); out2 += same when given
template <typename R>
__global__ void cay_combine_kernel(const cx<R> *__restrict__ V, long long n, const GmresState *__restrict__ st,
                                   cxd *__restrict__ out, cxd *__restrict__ out2)
{
    __shared__ cxd ys[GM_MAXM];
    const int k = st->stats.k;
    for (int j = threadIdx.x; j < k; j += blockDim.x) ys[j] = mk<double>(st->y[2 * j], st->y[2 * j + 1]);
    __syncthreads();
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x) {
        double ax = 0.0, ay = 0.0;
        for (int j = 0; j < k; ++j) {
            const cx<R> v = V[(size_t)j * n + i];
            const cxd q = ys[j];
            ax = fma((double)v.x, q.x, ax); ax = fma(-(double)v.y, q.y, ax);
            ay = fma((double)v.x, q.y, ay); ay = fma((double)v.y, q.x, ay);
        }
        out[i] = mk<double>(ax, ay);
        if (out2) out2[i] = out2[i] + mk<double>(ax, ay);
    }
}

__global__ void cay_true_resid_kernel(GmresState *st, double *nrm)
{
    if (threadIdx.x == 0 && blockIdx.x == 0) {
        st->stats.true_resid = sqrt(fmax(nrm[0], 0.0));
        nrm[0] = 0.0;
        nrm[1] = 0.0;
    }
}

// end of a refinement pass: record ||r|| (FP64) and repeat while it is above tol
__global__ void cay_refine_decide_kernel(GmresState *st, double *nrm, double tol, int maxpass,
                                         cudaGraphConditionalHandle outer, int use_cond)
{
    if (threadIdx.x != 0 || blockIdx.x != 0) return;
    const double r = sqrt(fmax(nrm[0], 0.0));
    nrm[0] = 0.0;
    nrm[1] = 0.0;
    st->stats.true_resid = r;
    const bool again = (r > tol) && (r == r) && st->stats.passes < maxpass;
    st->cont_outer = again ? 1 : 0;
    if (use_cond) cudaGraphSetConditional(outer, again ? 1u : 0u);
}

// Learned preconditioner application for flexible GMRES: z = y + s * (out_re + i out_im)
// with y = M^-1 V_j (in vcur), out the network's correction per block ([nblk][d_out]) and s
// the coupling's scale; the result goes to Z[j] (the flexible basis) and zcur (matvec source).
// With the learned part switched off for this step (st->learned_on == 0) z = y.
__global__ void cay_learned_apply_kernel(const GmresState *__restrict__ st, const cxf *__restrict__ y,
                                         const float *__restrict__ out, int N, int d_out,
                                         const cxd *__restrict__ s, cxf *__restrict__ Z, cxf *__restrict__ zcur,
                                         long long n)
{
    const int j = st->j;
    const bool on = st->learned_on != 0;
    const cxf sc = mk<float>((float)s->x, (float)s->y);
    cxf *Zj = Z + (size_t)j * n;
    for (long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x; e < n; e += (long long)gridDim.x * blockDim.x) {
        cxf v = y[e];
        if (on) {
            const long long a = e / N, i = e - a * N;
            const float ox = out[a * d_out + 2 * i], oy = out[a * d_out + 2 * i + 1];
            v.x += sc.x * ox - sc.y * oy;
            v.y += sc.x * oy + sc.y * ox;
        }
        Zj[e] = v;
        zcur[e] = v;
    }
}

// End of a learned pass: the candidate residual rn = r - A e (FP64) is judged against the
// pass's starting residual (beta0). A pass with the learned part that does not halve the
// residual (or gives a non-finite one) is discarded and the rest of the step runs with the
// block preconditioner alone. Decides whether another pass runs.
__global__ void cay_learned_decide_kernel(GmresState *st, double *nrm, double tol, int maxpass,
                                          cudaGraphConditionalHandle outer, int use_cond)
{
    if (threadIdx.x != 0 || blockIdx.x != 0) return;
    const double r = sqrt(fmax(nrm[0], 0.0));
    nrm[0] = 0.0;
    nrm[1] = 0.0;
    const double r0 = st->stats.beta0;
    bool accept = (r == r) && r < 1e300;
    if (accept && st->learned_on && !(r < 0.5 * r0)) accept = false;
    if (!accept && st->learned_on) {
        st->learned_on = 0;
        st->stats.rejected += 1;
    }
    st->accept = accept ? 1 : 0;
    const double rc = accept ? r : r0;
    st->stats.true_resid = rc;
    const bool again = (rc > tol) && (rc == rc) && st->stats.passes < maxpass;
    st->cont_outer = again ? 1 : 0;
    if (use_cond) cudaGraphSetConditional(outer, again ? 1u : 0u);
}

// psi += e and r = rn when the pass was accepted
__global__ void cay_learned_commit_kernel(const GmresState *__restrict__ st, const cxd *__restrict__ e,
                                          const cxd *__restrict__ rn, cxd *__restrict__ psi, cxd *__restrict__ r,
                                          long long n)
{
    if (!st->accept) return;
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x) {
        psi[i] = psi[i] + e[i];
        r[i] = rn[i];
    }
}

// ------------------------------------------------------------------------------------
// host object
// ------------------------------------------------------------------------------------
struct pg_cayley {
    pg_op *op64 = nullptr, *opb = nullptr;
    pg_banded *prec64 = nullptr, *precb = nullptr;
    pg_ctx *ctx = nullptr;
    pg_ctx rctx;                      // private reduction scratch: steppers may run concurrently
    StepParams *params_dev = nullptr; // where the graph reads this step's parameters
    int m = 0, prec = PG_FP64;
    long long n = 0;
    double tol = 1e-13;
    int true_residual = 0;
    void *V = nullptr, *w = nullptr, *vcur = nullptr, *dconv = nullptr;
    cxd *b64 = nullptr, *r64 = nullptr, *d64 = nullptr, *e64 = nullptr;
    double *h1 = nullptr, *h2 = nullptr, *h3 = nullptr, *nrm = nullptr, *nrm2 = nullptr;
    GmresState *st = nullptr;
    GmresStats *h_stats = nullptr;    // mapped pinned host memory (the single-kernel step writes it)
    int *h_err = nullptr;             // the context's device error word after the last step (mapped)
    GmresStats *dm_stats = nullptr;   // device-visible aliases of h_stats and h_err
    int *dm_err = nullptr;
    StepParams *d_params = nullptr;
    StepParams *h_ring = nullptr;
    cudaEvent_t ring_ev[RING];
    bool ring_used[RING];
    int ring_pos = 0;
    cxd *d_sc = nullptr;
    cudaGraph_t graph = nullptr;
    cudaGraphExec_t exec = nullptr;
    void *built_psi = nullptr;
    cudaStream_t cap[3] = {nullptr, nullptr, nullptr};
    bool eager = false;  // host-driven loops (same kernels; for profilers that cannot see graph loops)
    int h_flag = 0;
    long long kernels_counted = 0;  // device kernel count already added to ctx->launches
    // learned preconditioner (mixed precision only)
    pg_mlp *mlp = nullptr;
    int learned_slot = 0;          // operator slot whose scale i dt/2 h(t) multiplies the correction
    void *Z = nullptr, *zcur = nullptr, *Xf = nullptr;
    float *mlp_out = nullptr;
    cxd *rn64 = nullptr;
    // single-kernel mixed step (cayley_fused.cu), when the operators qualify
    FusedCayley *fused = nullptr;
    int fused_status = PG_ERR_STATE;  // why the single-kernel step is unavailable (PG_OK: it is)
    bool use_fused = true;
};

static int nblocks_for(pg_ctx *ctx, long long n)
{
    return (int)std::max<long long>(1, std::min<long long>((n + 255) / 256, 4LL * std::max(1, ctx->num_sms)));
}

// Conditional handle on the graph being captured by stream s.
static int capture_handle(cudaStream_t s, cudaGraphConditionalHandle *handle, unsigned def, unsigned flags)
{
    cudaStreamCaptureStatus status;
    cudaGraph_t g;
    PG_CUDA_TRY(cudaStreamGetCaptureInfo(s, &status, nullptr, &g, nullptr, nullptr, nullptr));
    if (status != cudaStreamCaptureStatusActive) return PG_ERR_STATE;
    PG_CUDA_TRY(cudaGraphConditionalHandleCreate(handle, g, def, flags));
    return PG_OK;
}

// WHILE node on `handle` appended to the capture of stream s; its body graph in *body.
static int capture_while(cudaStream_t s, cudaGraphConditionalHandle handle, cudaGraph_t *body)
{
    cudaStreamCaptureStatus status;
    cudaGraph_t g;
    const cudaGraphNode_t *deps = nullptr;
    size_t ndeps = 0;
    PG_CUDA_TRY(cudaStreamGetCaptureInfo(s, &status, nullptr, &g, &deps, nullptr, &ndeps));
    if (status != cudaStreamCaptureStatusActive) return PG_ERR_STATE;
    cudaGraphNodeParams p = {cudaGraphNodeTypeConditional};
    p.conditional.handle = handle;
    p.conditional.type = cudaGraphCondTypeWhile;
    p.conditional.size = 1;
    cudaGraphNode_t node;
    PG_CUDA_TRY(cudaGraphAddNode(&node, g, deps, nullptr, ndeps, &p));
    *body = p.conditional.phGraph_out[0];
    PG_CUDA_TRY(cudaStreamUpdateCaptureDependencies(s, &node, nullptr, 1, cudaStreamSetCaptureDependencies));
    return PG_OK;
}

// kernels of one GMRES iteration, captured on ctx->stream
template <typename R, typename T>
static int capture_iteration(pg_cayley *c, pg_op *op, pg_banded *pre, cudaGraphConditionalHandle inner)
{
    pg_ctx *ctx = c->ctx;
    cudaStream_t s = ctx->stream;
    const long long n = c->n;
    const int nb = nblocks_for(ctx, n);
    cx<R> *V = (cx<R> *)c->V, *w = (cx<R> *)c->w, *vcur = (cx<R> *)c->vcur;
    cay_next_vector_kernel<R><<<nb, 256, 0, s>>>(c->st, V, w, vcur, n);
    PG_TRY(pg_check_launch(ctx));
    pg_scales dummy;
    memset(&dummy, 0, sizeof(dummy));
    PG_TRY(pg_op_matvec_dev(op, dummy, c->d_sc + SC_PLUS * PG_MAX_SLOTS, vcur, w, 0, nullptr, nullptr));
    PG_TRY(pg_banded_apply_dev(pre, PG_BAND_PREC_SOLVE, w));
    pg_ctx *rc = &c->rctx;
    rc->stream = s;
    // reductions add into h1/h2/h3 with FP64 atomics; the Givens kernel reads and clears them
    PG_TRY(pg_multidot<R>(rc, V, n, c->m, w, n, c->h1, &c->st->j, 1));
    PG_TRY(pg_gs_update<R>(rc, V, n, c->m, c->h1, w, n, 1, c->h2, &c->st->j, 1));
    PG_TRY(pg_gs_update<R>(rc, V, n, c->m, c->h2, w, n, 0, c->h3, &c->st->j, 1));
    cay_gmres_finalize_kernel<T><<<1, 32, 0, s>>>(c->st, c->h1, c->h2, c->h3, c->m, inner, c->eager ? 0 : 1,
                                                   K_ITER - 2 + pg_op_matvec_kernels(op) + pg_banded_solve_kernels(pre));
    return pg_check_launch(ctx);
}

// kernels of one flexible GMRES iteration with the learned preconditioner (complex64):
// y = M^-1 V_j, z_j = y + s MLP(features(y)), w = A z_j, then the same orthogonalization and
// Givens update as capture_iteration
static int capture_iteration_learned(pg_cayley *c, cudaGraphConditionalHandle inner)
{
    pg_ctx *ctx = c->ctx;
    cudaStream_t s = ctx->stream;
    const long long n = c->n;
    const int nb = nblocks_for(ctx, n);
    cxf *V = (cxf *)c->V, *w = (cxf *)c->w, *vcur = (cxf *)c->vcur;
    cay_next_vector_kernel<float><<<nb, 256, 0, s>>>(c->st, V, w, vcur, n);
    PG_TRY(pg_check_launch(ctx));
    PG_TRY(pg_banded_apply_dev(c->precb, PG_BAND_PREC_SOLVE, vcur));
    pg_ctx *mctx = nullptr;
    int d_in = 0, d_out = 0;
    PG_TRY(pg_mlp_describe(c->mlp, &mctx, &d_in, &d_out));
    // one network row per angular channel; a channel's block is [N] (one electron) or [N][N]
    const int nblk = c->opb->shape[0], N = (int)(c->n / nblk);
    PG_TRY(pg_mlp_block_features_dev(ctx, vcur, nblk, N, d_in, nullptr, c->Xf));
    PG_TRY(pg_mlp_forward_dev(c->mlp, c->Xf, nblk, c->mlp_out));
    cay_learned_apply_kernel<<<nb, 256, 0, s>>>(c->st, vcur, c->mlp_out, N, d_out,
                                                c->d_sc + SC_PLUS * PG_MAX_SLOTS + c->learned_slot, (cxf *)c->Z,
                                                (cxf *)c->zcur, n);
    PG_TRY(pg_check_launch(ctx));
    pg_scales dummy;
    memset(&dummy, 0, sizeof(dummy));
    PG_TRY(pg_op_matvec_dev(c->opb, dummy, c->d_sc + SC_PLUS * PG_MAX_SLOTS, c->zcur, w, 0, nullptr, nullptr));
    pg_ctx *rc = &c->rctx;
    rc->stream = s;
    PG_TRY(pg_multidot<float>(rc, V, n, c->m, w, n, c->h1, &c->st->j, 1));
    PG_TRY(pg_gs_update<float>(rc, V, n, c->m, c->h1, w, n, 1, c->h2, &c->st->j, 1));
    PG_TRY(pg_gs_update<float>(rc, V, n, c->m, c->h2, w, n, 0, c->h3, &c->st->j, 1));
    cay_gmres_finalize_kernel<float><<<1, 32, 0, s>>>(c->st, c->h1, c->h2, c->h3, c->m, inner, c->eager ? 0 : 1,
                                                      K_LEARN_ITER - 2 + pg_op_matvec_kernels(c->opb) +
                                                          pg_banded_solve_kernels(c->precb));
    return pg_check_launch(ctx);
}

// WHILE loop: a conditional graph node whose body `fn` records on `body_stream`, or, in the
// eager mode, a host loop on the current stream reading the device flag `flag`.
template <typename F>
static int loop_while(pg_cayley *c, cudaGraphConditionalHandle handle, cudaStream_t body_stream, const int *flag, F fn)
{
    pg_ctx *ctx = c->ctx;
    if (!c->eager) {
        cudaGraph_t body;
        PG_TRY(capture_while(ctx->stream, handle, &body));
        return capture_body(c, body_stream, body, fn);
    }
    for (int guard = 0; guard < 1000; ++guard) {
        int v = 0;
        PG_CUDA_TRY(cudaMemcpyAsync(&c->h_flag, flag, sizeof(int), cudaMemcpyDeviceToHost, ctx->stream));
        PG_CUDA_TRY(cudaStreamSynchronize(ctx->stream));
        v = c->h_flag;
        if (!v) return PG_OK;
        PG_TRY(fn());
    }
    return PG_ERR_NOT_CONVERGED;
}

// Capture a nested body: begin capture of stream s into `body`, run fn with ctx->stream = s.
template <typename F>
static int capture_body(pg_cayley *c, cudaStream_t s, cudaGraph_t body, F fn)
{
    pg_ctx *ctx = c->ctx;
    PG_CUDA_TRY(cudaStreamBeginCaptureToGraph(s, body, nullptr, nullptr, 0, cudaStreamCaptureModeThreadLocal));
    cudaStream_t saved = ctx->stream;
    ctx->stream = s;
    int code = fn();
    ctx->stream = saved;
    cudaGraph_t out = nullptr;
    cudaError_t e = cudaStreamEndCapture(s, &out);
    if (code == PG_OK && e != cudaSuccess) {
        pg_set_last_error(e, "cudaStreamEndCapture(body)", __FILE__, __LINE__);
        code = PG_ERR_CUDA;
    }
    return code;
}

// plain FP64 step (the reference scheme)
static int record_fp64(pg_cayley *c, cxd *psi)
{
    pg_ctx *ctx = c->ctx;
    cudaStream_t s0 = ctx->stream;
    const long long n = c->n;
    const int nb = nblocks_for(ctx, n);
    pg_scales dummy;
    memset(&dummy, 0, sizeof(dummy));
    pg_ctx *rc = &c->rctx;
    rc->stream = s0;
    const int mv = pg_op_matvec_kernels(c->op64) - 1;
    cay_scales_kernel<<<1, 32, 0, s0>>>(c->params_dev, c->d_sc, c->st,
                                        K_FP64_BASE + mv + pg_banded_solve_kernels(c->prec64) - 1 +
                                            (c->true_residual ? K_TRUE_RESID + mv : 0));
    PG_TRY(pg_check_launch(ctx));
    PG_TRY(pg_op_matvec_dev(c->op64, dummy, c->d_sc + SC_MINUS * PG_MAX_SLOTS, psi, c->b64, 0, nullptr, nullptr));
    PG_CUDA_TRY(cudaMemcpyAsync(c->d64, c->b64, sizeof(cxd) * n, cudaMemcpyDeviceToDevice, s0));
    PG_TRY(pg_banded_apply_dev(c->prec64, PG_BAND_PREC_SOLVE, c->d64));
    PG_TRY(pg_multidot<double>(rc, c->d64, n, 0, c->d64, n, c->nrm, nullptr, 1));
    cudaGraphConditionalHandle inner = 0;
    if (!c->eager) PG_TRY(capture_handle(s0, &inner, 0, 0));
    cay_gmres_init_kernel<double><<<nb, 256, 0, s0>>>(c->st, c->nrm, c->d64, (cxd *)c->V, (cxd *)c->vcur, n, c->tol,
                                                      0.0, 0, inner, inner, c->eager ? -1 : 0);
    PG_TRY(pg_check_launch(ctx));
    PG_TRY(loop_while(c, inner, c->cap[1], &c->st->cont_inner,
                      [&]() { return capture_iteration<double, double>(c, c->op64, c->prec64, inner); }));
    cay_backsolve_kernel<double><<<1, 32, 0, s0>>>(c->st, c->nrm);
    PG_TRY(pg_check_launch(ctx));
    cay_combine_kernel<double><<<nb, 256, 0, s0>>>((const cxd *)c->V, n, c->st, psi, nullptr);
    PG_TRY(pg_check_launch(ctx));
    if (c->true_residual) {
        // ||(S + i dt/2 H) psi' - b||
        PG_TRY(pg_op_matvec_dev(c->op64, dummy, c->d_sc + SC_PLUS * PG_MAX_SLOTS, psi, c->r64, 0, nullptr, nullptr));
        PG_TRY(pg_axpy(ctx, mk<double>(-1.0, 0.0), c->b64, c->r64, n));
        rc->stream = s0;
        PG_TRY(pg_multidot<double>(rc, c->r64, n, 0, c->r64, n, c->nrm2, nullptr, 1));
        cay_true_resid_kernel<<<1, 32, 0, s0>>>(c->st, c->nrm2);
        PG_TRY(pg_check_launch(ctx));
    }
    PG_CUDA_TRY(cudaMemcpyAsync(c->h_stats, &c->st->stats, sizeof(GmresStats), cudaMemcpyDeviceToHost, s0));
    return PG_OK;
}

// mixed step: FP64 residual, complex64 GMRES correction, refinement WHILE loop that
// repeats while the FP64 true residual ||b - A psi|| is above tol (at most 4 passes)
static int record_mixed(pg_cayley *c, cxd *psi)
{
    pg_ctx *ctx = c->ctx;
    cudaStream_t s0 = ctx->stream;
    const long long n = c->n;
    const int nb = nblocks_for(ctx, n);
    pg_scales dummy;
    memset(&dummy, 0, sizeof(dummy));
    pg_ctx *rc = &c->rctx;
    const int mv = pg_op_matvec_kernels(c->op64) - 1;
    cay_scales_kernel<<<1, 32, 0, s0>>>(c->params_dev, c->d_sc, c->st, K_MIXED_BASE + mv);
    PG_TRY(pg_check_launch(ctx));
    PG_TRY(pg_op_matvec_dev(c->op64, dummy, c->d_sc + SC_DIFF * PG_MAX_SLOTS, psi, c->r64, 0, nullptr, nullptr));
    cudaGraphConditionalHandle outer = 0;
    if (!c->eager) {
        PG_TRY(capture_handle(s0, &outer, 1, cudaGraphCondAssignDefault));
    } else {
        PG_CUDA_TRY(cudaMemsetAsync(&c->st->cont_outer, 0xff, sizeof(int), s0));  // first pass always runs
    }
    const bool learned = c->mlp != nullptr;
    PG_TRY(loop_while(c, outer, c->cap[1], &c->st->cont_outer, [&]() -> int {
        cudaStream_t s1 = ctx->stream;
        cxf *dconv = (cxf *)c->dconv;
        PG_TRY((pg_scale_copy<float, double>(ctx, c->r64, dconv, nullptr, n, nullptr, 1.0)));
        // left preconditioning solves M^-1 A e = M^-1 r; the learned (flexible, right)
        // variant solves A P e' = r, its residual estimate being the true residual's
        if (!learned) PG_TRY(pg_banded_apply_dev(c->precb, PG_BAND_PREC_SOLVE, dconv));
        rc->stream = s1;
        PG_TRY(pg_multidot<float>(rc, dconv, n, 0, dconv, n, c->nrm, nullptr, 1));
        cudaGraphConditionalHandle inner = 0;
        if (!c->eager) PG_TRY(capture_handle(s1, &inner, 0, 0));
        cay_gmres_init_kernel<float><<<nb, 256, 0, s1>>>(c->st, c->nrm, dconv, (cxf *)c->V, (cxf *)c->vcur, n, c->tol,
                                                         2e-6, (learned ? K_LEARN_PASS : K_MIXED_PASS + pg_banded_solve_kernels(c->precb) - 1) + mv,
                                                         inner, outer,
                                                         c->eager ? -1 : 1);
        PG_TRY(pg_check_launch(ctx));
        PG_TRY(loop_while(c, inner, c->cap[2], &c->st->cont_inner, [&]() {
            return learned ? capture_iteration_learned(c, inner)
                           : capture_iteration<float, float>(c, c->opb, c->precb, inner);
        }));
        cay_backsolve_kernel<float><<<1, 32, 0, s1>>>(c->st, c->nrm);
        PG_TRY(pg_check_launch(ctx));
        if (learned) {
            // e = Z y; rn = r - A e; judged, then committed or discarded
            cay_combine_kernel<float><<<nb, 256, 0, s1>>>((const cxf *)c->Z, n, c->st, c->e64, nullptr);
            PG_TRY(pg_check_launch(ctx));
            PG_CUDA_TRY(cudaMemcpyAsync(c->rn64, c->r64, sizeof(cxd) * n, cudaMemcpyDeviceToDevice, s1));
            PG_TRY(pg_op_matvec_dev(c->op64, dummy, c->d_sc + SC_NEGPLUS * PG_MAX_SLOTS, c->e64, c->rn64, 1, nullptr,
                                    nullptr));
            rc->stream = s1;
            PG_TRY(pg_multidot<double>(rc, c->rn64, n, 0, c->rn64, n, c->nrm2, nullptr, 1));
            cay_learned_decide_kernel<<<1, 32, 0, s1>>>(c->st, c->nrm2, c->tol, 4, outer, c->eager ? 0 : 1);
            PG_TRY(pg_check_launch(ctx));
            cay_learned_commit_kernel<<<nb, 256, 0, s1>>>(c->st, c->e64, c->rn64, psi, c->r64, n);
            return pg_check_launch(ctx);
        }
        cay_combine_kernel<float><<<nb, 256, 0, s1>>>((const cxf *)c->V, n, c->st, c->e64, psi);
        PG_TRY(pg_check_launch(ctx));
        // r -= (S + i dt/2 H) e   in FP64, then ||r|| decides whether another pass runs
        PG_TRY(pg_op_matvec_dev(c->op64, dummy, c->d_sc + SC_NEGPLUS * PG_MAX_SLOTS, c->e64, c->r64, 1, nullptr, nullptr));
        rc->stream = s1;
        PG_TRY(pg_multidot<double>(rc, c->r64, n, 0, c->r64, n, c->nrm2, nullptr, 1));
        cay_refine_decide_kernel<<<1, 32, 0, s1>>>(c->st, c->nrm2, c->tol, 4, outer, c->eager ? 0 : 1);
        return pg_check_launch(ctx);
    }));
    PG_CUDA_TRY(cudaMemcpyAsync(c->h_stats, &c->st->stats, sizeof(GmresStats), cudaMemcpyDeviceToHost, s0));
    return PG_OK;
}

static int build_graph(pg_cayley *c, cxd *psi)
{
    pg_ctx *ctx = c->ctx;
    if (c->exec) { cudaGraphExecDestroy(c->exec); c->exec = nullptr; }
    if (c->graph) { cudaGraphDestroy(c->graph); c->graph = nullptr; }
    cudaStream_t saved = ctx->stream;
    PG_CUDA_TRY(cudaStreamBeginCapture(c->cap[0], cudaStreamCaptureModeThreadLocal));
    ctx->stream = c->cap[0];
    int code = (c->prec == PG_FP64) ? record_fp64(c, psi) : record_mixed(c, psi);
    ctx->stream = saved;
    cudaGraph_t g = nullptr;
    cudaError_t e = cudaStreamEndCapture(c->cap[0], &g);
    if (code != PG_OK) {
        if (g) cudaGraphDestroy(g);
        return code;
    }
    if (e != cudaSuccess) {
        pg_set_last_error(e, "cudaStreamEndCapture", __FILE__, __LINE__);
        return PG_ERR_CUDA;
    }
    c->graph = g;
    PG_CUDA_TRY(cudaGraphInstantiate(&c->exec, g, 0));
    c->built_psi = psi;
    return PG_OK;
}

extern "C" int pg_cayley_create(pg_op *op64, pg_op *op_basis, pg_banded *prec64, pg_banded *prec_basis, int basis_size,
                                int basis_precision, double tolerance, pg_cayley **out)
{
    if (!op64 || !op_basis || !prec64 || !prec_basis || !out) return PG_ERR_ARG;
    if (basis_size < 2 || basis_size > GM_MAXM || basis_size > PG_RED_COLS - 2) return PG_ERR_ARG;
    if (op64->precision != PG_FP64 || op_basis->precision != basis_precision) return PG_ERR_ARG;
    if (prec64->kind < 1 || prec64->kind > 3 || prec_basis->kind < 1 || prec_basis->kind > 3) return PG_ERR_ARG;
    if (prec64->op->precision != PG_FP64 || prec_basis->op->precision != basis_precision) return PG_ERR_ARG;
    if (basis_precision != PG_FP64 && basis_precision != PG_FP32) return PG_ERR_ARG;
    pg_cayley *c = new pg_cayley();
    c->op64 = op64;
    c->opb = op_basis;
    c->prec64 = prec64;
    c->precb = prec_basis;
    c->ctx = op64->ctx;
    c->m = basis_size;
    c->prec = basis_precision;
    c->tol = std::max(tolerance, 1e-13);
    c->n = (long long)op64->nrows * op64->N;
    const size_t esz = basis_precision == PG_FP64 ? sizeof(cxd) : sizeof(cxf);
    PG_CUDA_TRY(cudaMalloc(&c->V, esz * (size_t)c->m * c->n));
    PG_CUDA_TRY(cudaMalloc(&c->w, esz * (size_t)c->n));
    PG_CUDA_TRY(cudaMalloc(&c->vcur, esz * (size_t)c->n));
    PG_CUDA_TRY(cudaMalloc(&c->dconv, esz * (size_t)c->n));
    PG_CUDA_TRY(cudaMalloc(&c->b64, sizeof(cxd) * (size_t)c->n));
    PG_CUDA_TRY(cudaMalloc(&c->r64, sizeof(cxd) * (size_t)c->n));
    PG_CUDA_TRY(cudaMalloc(&c->d64, sizeof(cxd) * (size_t)c->n));
    PG_CUDA_TRY(cudaMalloc(&c->e64, sizeof(cxd) * (size_t)c->n));
    const size_t cols = sizeof(double) * 2 * (PG_RED_COLS + 2);
    PG_CUDA_TRY(cudaMalloc(&c->h1, cols));
    PG_CUDA_TRY(cudaMalloc(&c->h2, cols));
    PG_CUDA_TRY(cudaMalloc(&c->h3, cols));
    PG_CUDA_TRY(cudaMalloc(&c->nrm, cols));
    PG_CUDA_TRY(cudaMalloc(&c->nrm2, cols));
    // atomic reduction targets start (and are left by their consumers) at zero
    for (double *z : {c->h1, c->h2, c->h3, c->nrm, c->nrm2}) PG_CUDA_TRY(cudaMemset(z, 0, cols));
    PG_CUDA_TRY(cudaMalloc(&c->st, sizeof(GmresState)));
    PG_CUDA_TRY(cudaMemset(c->st, 0, sizeof(GmresState)));
    PG_CUDA_TRY(cudaHostAlloc(&c->h_stats, sizeof(GmresStats), cudaHostAllocMapped));
    memset(c->h_stats, 0, sizeof(GmresStats));
    PG_CUDA_TRY(cudaHostAlloc(&c->h_err, sizeof(int), cudaHostAllocMapped));
    *c->h_err = 0;
    PG_CUDA_TRY(cudaHostGetDevicePointer((void **)&c->dm_stats, c->h_stats, 0));
    PG_CUDA_TRY(cudaHostGetDevicePointer((void **)&c->dm_err, c->h_err, 0));
    PG_CUDA_TRY(cudaMalloc(&c->d_params, sizeof(StepParams)));
    c->params_dev = c->d_params;
    c->rctx.device = c->ctx->device;
    c->rctx.num_sms = c->ctx->num_sms;
    c->rctx.stream = c->ctx->stream;
    PG_TRY(pg_ctx_ensure_reduction(&c->rctx));
    PG_CUDA_TRY(cudaMallocHost(&c->h_ring, sizeof(StepParams) * RING));
    PG_CUDA_TRY(cudaMalloc(&c->d_sc, sizeof(cxd) * SC_COUNT * PG_MAX_SLOTS));
    for (int k = 0; k < RING; ++k) {
        PG_CUDA_TRY(cudaEventCreateWithFlags(&c->ring_ev[k], cudaEventDisableTiming));
        c->ring_used[k] = false;
    }
    for (int k = 0; k < 3; ++k) PG_CUDA_TRY(cudaStreamCreateWithFlags(&c->cap[k], cudaStreamNonBlocking));
    // rank-2 banded operators with the block LU preconditioner run the mixed step as one
    // kernel; anything else (or a failed check) keeps the captured multi-kernel step
    if (basis_precision == PG_FP32) {
        c->fused_status = pg_cayley_fused_prepare(op64, op_basis, prec_basis, c->m, &c->fused);
        if (c->fused_status != PG_OK) {
            c->fused = nullptr;
            cudaGetLastError();
        }
    }
    *out = c;
    return PG_OK;
}

extern "C" int pg_cayley_destroy(pg_cayley *c)
{
    if (!c) return PG_ERR_ARG;
    cudaStreamSynchronize(c->ctx->stream);
    if (c->exec) cudaGraphExecDestroy(c->exec);
    if (c->graph) cudaGraphDestroy(c->graph);
    for (int k = 0; k < 3; ++k)
        if (c->cap[k]) cudaStreamDestroy(c->cap[k]);
    for (int k = 0; k < RING; ++k) cudaEventDestroy(c->ring_ev[k]);
    pg_cayley_fused_free(c->fused);
    for (void *p : {c->Z, c->zcur, c->Xf, (void *)c->mlp_out, (void *)c->rn64}) cudaFree(p);
    void *bufs[] = {c->V, c->w, c->vcur, c->dconv, c->b64, c->r64, c->d64, c->e64, c->h1, c->h2, c->h3, c->nrm,
                    c->nrm2, c->st, c->d_params, c->d_sc, c->rctx.red_partial, c->rctx.red_counter,
                    c->rctx.red_out, c->rctx.d_err};
    for (void *b : bufs) cudaFree(b);
    if (c->rctx.h_pinned) cudaFreeHost(c->rctx.h_pinned);
    if (c->h_stats) cudaFreeHost(c->h_stats);
    if (c->h_err) cudaFreeHost(c->h_err);
    if (c->h_ring) cudaFreeHost(c->h_ring);
    delete c;
    return PG_OK;
}

// one step: upload this step's H(t+dt/2) slot values, launch the graph (or, in the eager
// mode, run the same kernels with the loops on the host)
static int cayley_launch(pg_cayley *c, cxd *psi, double dt, const double *scales, int nscales)
{
    pg_ctx *ctx = c->ctx;
    // kernels are counted on the device (GmresStats::kernels), not while recording
    const long long launches = ctx->launches;
    const bool fused = c->fused && c->use_fused && !c->mlp && !c->eager;
    if (!fused && !c->eager && (!c->exec || c->built_psi != psi)) {
        const int code = build_graph(c, psi);
        ctx->launches = launches;
        PG_TRY(code);
    }
    if (fused) {
        // the step's parameters as kernel arguments; statistics and the error word come back
        // through mapped host memory written by the kernel
        StepParams p;
        memset(&p, 0, sizeof(p));
        p.dt = dt;
        for (int k = 0; k < PG_MAX_SLOTS; ++k)
            p.h[k] = mk<double>(k < nscales ? scales[2 * k] : 0.0, k < nscales ? scales[2 * k + 1] : 0.0);
        return pg_cayley_fused_launch(c->fused, ctx->stream, p, psi, c->st, c->tol, ctx->d_err, c->dm_stats, c->dm_err);
    }
    const int slot = c->ring_pos;
    c->ring_pos = (c->ring_pos + 1) % RING;
    if (c->ring_used[slot]) PG_CUDA_TRY(cudaEventSynchronize(c->ring_ev[slot]));
    StepParams &p = c->h_ring[slot];
    memset(&p, 0, sizeof(p));
    p.dt = dt;
    for (int k = 0; k < PG_MAX_SLOTS; ++k) p.h[k] = mk<double>(k < nscales ? scales[2 * k] : 0.0, k < nscales ? scales[2 * k + 1] : 0.0);
    PG_CUDA_TRY(cudaMemcpyAsync(c->d_params, &p, sizeof(StepParams), cudaMemcpyHostToDevice, ctx->stream));
    PG_CUDA_TRY(cudaEventRecord(c->ring_ev[slot], ctx->stream));
    c->ring_used[slot] = true;
    if (c->eager) {
        c->rctx.stream = ctx->stream;
        const int code = (c->prec == PG_FP64) ? record_fp64(c, psi) : record_mixed(c, psi);
        ctx->launches = launches;
        PG_TRY(code);
    } else {
        PG_CUDA_TRY(cudaGraphLaunch(c->exec, ctx->stream));
    }
    // the error word is sticky (until pg_ctx_clear_device_error): read after the step, it says
    // whether a bounded wait of this step, or of an earlier one, ran out
    PG_CUDA_TRY(cudaMemcpyAsync(c->h_err, ctx->d_err, sizeof(int), cudaMemcpyDeviceToHost, ctx->stream));
    return PG_OK;
}

// statistics of the last completed step; adds the kernels run since the last call to the
// context's launch count. PG_ERR_NOT_CONVERGED when a step was abandoned: the context's device
// error word was set when the last step ended (a bounded wait of that step or of an earlier one
// since the word was last cleared ran out; the word says which kind), or no refinement pass
// started. A single-kernel step abandoned at its first grid barrier leaves psi unchanged; one
// abandoned later may have left psi partly corrected.
static int fill_stats(pg_cayley *c, pg_krylov_stats *st)
{
    const GmresStats &g = *c->h_stats;
    c->ctx->launches += g.kernels - c->kernels_counted;
    c->kernels_counted = g.kernels;
    st->Iterations = g.iterations;
    st->OpCount = g.iterations;
    st->InnerProductCount = 2 * g.iterations;
    st->ReOrthoCount = g.iterations;
    st->RestartCount = g.passes;
    st->ErrorEstimate = g.resid;
    st->TrueResidual = g.true_resid;
    return (g.passes > 0 && *c->h_err == 0) ? PG_OK : PG_ERR_NOT_CONVERGED;
}

extern "C" int pg_cayley_step(pg_cayley *c, void *psi, double dt, const double *scales, int nscales, pg_krylov_stats *st)
{
    if (!c || !psi || !scales || nscales < 1 || nscales > PG_MAX_SLOTS) return PG_ERR_ARG;
    PG_TRY(cayley_launch(c, (cxd *)psi, dt, scales, nscales));
    if (st) {
        PG_CUDA_TRY(cudaStreamSynchronize(c->ctx->stream));
        return fill_stats(c, st);
    }
    return PG_OK;
}

// Learned preconditioner for the mixed-precision step (nullptr switches it off). The
// correction is scaled by the slot's i dt/2 h(t); the network must take d_in >= 6N and give
// d_out >= 2N per angular block.
extern "C" int pg_cayley_set_learned(pg_cayley *c, pg_mlp *mlp, int coupling_slot)
{
    if (!c || coupling_slot < 0 || coupling_slot >= PG_MAX_SLOTS) return PG_ERR_ARG;
    if (!mlp) {
        c->mlp = nullptr;
        c->built_psi = nullptr;
        return PG_OK;
    }
    if (c->prec != PG_FP32) return PG_ERR_STATE;
    pg_ctx *mctx = nullptr;
    int d_in = 0, d_out = 0;
    PG_TRY(pg_mlp_describe(mlp, &mctx, &d_in, &d_out));
    const int nblk = c->opb->shape[0], N = (int)(c->n / nblk);
    if (mctx != c->ctx) return PG_ERR_ARG;
    if (d_in < 6 * N || d_out < 2 * N) return PG_ERR_SHAPE;
    PG_TRY(pg_mlp_reserve(mlp, nblk));
    cudaFree(c->Z); cudaFree(c->zcur); cudaFree(c->Xf); cudaFree(c->mlp_out); cudaFree(c->rn64);
    c->Z = c->zcur = c->Xf = nullptr;
    c->mlp_out = nullptr;
    c->rn64 = nullptr;
    PG_CUDA_TRY(cudaMalloc(&c->Z, sizeof(cxf) * (size_t)c->m * c->n));
    PG_CUDA_TRY(cudaMalloc(&c->zcur, sizeof(cxf) * (size_t)c->n));
    PG_CUDA_TRY(cudaMalloc(&c->Xf, 2 * (size_t)nblk * d_in));
    PG_CUDA_TRY(cudaMalloc(&c->mlp_out, sizeof(float) * (size_t)nblk * d_out));
    PG_CUDA_TRY(cudaMalloc(&c->rn64, sizeof(cxd) * (size_t)c->n));
    c->mlp = mlp;
    c->learned_slot = coupling_slot;
    c->built_psi = nullptr;  // rebuild the step graph
    return PG_OK;
}

// passes of the learned preconditioner rejected by the residual test so far (waits)
extern "C" int pg_cayley_learned_rejected(pg_cayley *c, long long *out)
{
    if (!c || !out) return PG_ERR_ARG;
    PG_CUDA_TRY(cudaStreamSynchronize(c->ctx->stream));
    *out = c->h_stats->rejected;
    return PG_OK;
}

extern "C" int pg_cayley_set_eager(pg_cayley *c, int on)
{
    if (!c) return PG_ERR_ARG;
    c->eager = on != 0;
    return PG_OK;
}

// Single-kernel mixed step on (the default where the operators qualify) or off (the
// captured multi-kernel step). Switching it on for a stepper that does not qualify returns
// the reason (PG_ERR_STATE: not a mixed-precision stepper; PG_ERR_STORAGE: operator or
// preconditioner kind; PG_ERR_SHAPE: basis size, fibre length or channel count).
extern "C" int pg_cayley_set_fused(pg_cayley *c, int on)
{
    if (!c) return PG_ERR_ARG;
    if (on && !c->fused) return c->fused_status != PG_OK ? c->fused_status : PG_ERR_STATE;
    c->use_fused = on != 0;
    return PG_OK;
}

extern "C" int pg_cayley_set_fused_variant(pg_cayley *c, int variant)
{
    if (!c) return PG_ERR_ARG;
    if (!c->fused) return c->fused_status != PG_OK ? c->fused_status : PG_ERR_STATE;
    return pg_cayley_fused_select(c->fused, variant);
}

extern "C" int pg_cayley_get_fused_variant(pg_cayley *c, int *variant)
{
    if (!c || !variant) return PG_ERR_ARG;
    *variant = (c->fused && c->use_fused && !c->mlp && !c->eager) ? pg_cayley_fused_which(c->fused) : 0;
    return PG_OK;
}

extern "C" int pg_cayley_set_barrier_probe(pg_cayley *c, int extra_arrivals, int at_barrier)
{
    if (!c || extra_arrivals < 0 || at_barrier < 0) return PG_ERR_ARG;
    if (!c->fused) return PG_ERR_STATE;
    pg_cayley_fused_set_probe(c->fused, (unsigned int)extra_arrivals, (unsigned int)at_barrier);
    return PG_OK;
}

extern "C" int pg_cayley_set_true_residual(pg_cayley *c, int on)
{
    if (!c) return PG_ERR_ARG;
    if ((on != 0) != (c->true_residual != 0)) {
        c->true_residual = on ? 1 : 0;
        c->built_psi = nullptr;  // rebuild the graph on the next step
    }
    return PG_OK;
}

extern "C" int pg_cayley_advance(pg_cayley *c, void *psi, double dt, int nsteps, const double *scales_table,
                                 int nscales, pg_krylov_stats *st)
{
    if (!c || !psi || !scales_table || nsteps < 0 || nscales < 1 || nscales > PG_MAX_SLOTS) return PG_ERR_ARG;
    long long iters = 0;
    for (int k = 0; k < nsteps; ++k)
        PG_TRY(cayley_launch(c, (cxd *)psi, dt, scales_table + 2 * (size_t)k * nscales, nscales));
    if (st) {
        PG_CUDA_TRY(cudaStreamSynchronize(c->ctx->stream));
        (void)iters;
        return fill_stats(c, st);
    }
    return PG_OK;
}

extern "C" int pg_cayley_last_stats(pg_cayley *c, pg_krylov_stats *st)
{
    if (!c || !st) return PG_ERR_ARG;
    PG_CUDA_TRY(cudaStreamSynchronize(c->ctx->stream));
    return fill_stats(c, st);
}

extern "C" int pg_cayley_totals(pg_cayley *c, long long *iterations, long long *passes)
{
    if (!c || !iterations || !passes) return PG_ERR_ARG;
    PG_CUDA_TRY(cudaStreamSynchronize(c->ctx->stream));
    *iterations = c->h_stats->cum_iterations;
    *passes = c->h_stats->cum_passes;
    return PG_OK;
}

// ------------------------------------------------------------------------------------
// ensembles: many independent Cayley steppers advanced by one graph launch
// ------------------------------------------------------------------------------------
// Each member keeps its own operator, preconditioner, Krylov basis, reduction scratch and
// conditional loops; the batch graph forks one branch per member from a common origin and
// joins them, so the members' kernels run concurrently and the whole ensemble step is a
// single cudaGraphLaunch. Step parameters of all members travel in one host-to-device copy.
struct pg_cayley_batch {
    std::vector<pg_cayley *> members;
    std::vector<void *> psis;
    pg_ctx *ctx = nullptr;
    StepParams *d_params = nullptr;
    StepParams *h_params = nullptr;
    cudaEvent_t params_done = nullptr;
    bool params_pending = false;
    cudaStream_t origin = nullptr;
    cudaEvent_t fork = nullptr;
    std::vector<cudaEvent_t> join;
    cudaGraph_t graph = nullptr;
    cudaGraphExec_t exec = nullptr;
};

extern "C" int pg_cayley_batch_create(pg_cayley **members, int nmembers, pg_cayley_batch **out)
{
    if (!members || nmembers < 1 || !out) return PG_ERR_ARG;
    pg_cayley_batch *b = new pg_cayley_batch();
    b->ctx = members[0]->ctx;
    for (int k = 0; k < nmembers; ++k) {
        if (!members[k] || members[k]->ctx != b->ctx) { delete b; return PG_ERR_ARG; }
        b->members.push_back(members[k]);
    }
    PG_CUDA_TRY(cudaMalloc(&b->d_params, sizeof(StepParams) * nmembers));
    PG_CUDA_TRY(cudaMallocHost(&b->h_params, sizeof(StepParams) * nmembers));
    memset(b->h_params, 0, sizeof(StepParams) * nmembers);
    PG_CUDA_TRY(cudaEventCreateWithFlags(&b->params_done, cudaEventDisableTiming));
    PG_CUDA_TRY(cudaStreamCreateWithFlags(&b->origin, cudaStreamNonBlocking));
    PG_CUDA_TRY(cudaEventCreateWithFlags(&b->fork, cudaEventDisableTiming));
    b->join.resize(nmembers);
    for (int k = 0; k < nmembers; ++k) PG_CUDA_TRY(cudaEventCreateWithFlags(&b->join[k], cudaEventDisableTiming));
    *out = b;
    return PG_OK;
}

extern "C" int pg_cayley_batch_destroy(pg_cayley_batch *b)
{
    if (!b) return PG_ERR_ARG;
    cudaStreamSynchronize(b->ctx->stream);
    if (b->exec) cudaGraphExecDestroy(b->exec);
    if (b->graph) cudaGraphDestroy(b->graph);
    for (auto e : b->join) cudaEventDestroy(e);
    cudaEventDestroy(b->fork);
    cudaEventDestroy(b->params_done);
    cudaStreamDestroy(b->origin);
    cudaFree(b->d_params);
    cudaFreeHost(b->h_params);
    for (pg_cayley *c : b->members) {
        c->params_dev = c->d_params;
        c->built_psi = nullptr;  // a member stepped alone again rebuilds its own graph
    }
    delete b;
    return PG_OK;
}

static int batch_build(pg_cayley_batch *b, void **psis)
{
    pg_ctx *ctx = b->ctx;
    if (b->exec) { cudaGraphExecDestroy(b->exec); b->exec = nullptr; }
    if (b->graph) { cudaGraphDestroy(b->graph); b->graph = nullptr; }
    const int n = (int)b->members.size();
    cudaStream_t saved = ctx->stream;
    PG_CUDA_TRY(cudaStreamBeginCapture(b->origin, cudaStreamCaptureModeThreadLocal));
    int code = PG_OK;
    if (cudaEventRecord(b->fork, b->origin) != cudaSuccess) code = PG_ERR_CUDA;
    for (int k = 0; k < n && code == PG_OK; ++k) {
        pg_cayley *c = b->members[k];
        c->params_dev = b->d_params + k;
        if (cudaStreamWaitEvent(c->cap[0], b->fork, 0) != cudaSuccess) { code = PG_ERR_CUDA; break; }
        ctx->stream = c->cap[0];
        code = (c->prec == PG_FP64) ? record_fp64(c, (cxd *)psis[k]) : record_mixed(c, (cxd *)psis[k]);
        ctx->stream = saved;
        if (code != PG_OK) break;
        if (cudaEventRecord(b->join[k], c->cap[0]) != cudaSuccess ||
            cudaStreamWaitEvent(b->origin, b->join[k], 0) != cudaSuccess)
            code = PG_ERR_CUDA;
    }
    ctx->stream = saved;
    cudaGraph_t g = nullptr;
    cudaError_t e = cudaStreamEndCapture(b->origin, &g);
    if (code != PG_OK) {
        if (g) cudaGraphDestroy(g);
        return code;
    }
    if (e != cudaSuccess) {
        pg_set_last_error(e, "cudaStreamEndCapture(batch)", __FILE__, __LINE__);
        return PG_ERR_CUDA;
    }
    b->graph = g;
    PG_CUDA_TRY(cudaGraphInstantiate(&b->exec, g, 0));
    b->psis.assign(psis, psis + n);
    for (pg_cayley *c : b->members) c->built_psi = nullptr;  // their own graphs no longer match
    return PG_OK;
}

// One ensemble step: member k's wavefunction psis[k], slot values scales[k][0..nscales).
extern "C" int pg_cayley_batch_step(pg_cayley_batch *b, void **psis, double dt, const double *scales, int nscales)
{
    if (!b || !psis || !scales || nscales < 1 || nscales > PG_MAX_SLOTS) return PG_ERR_ARG;
    const int n = (int)b->members.size();
    bool same = b->exec && (int)b->psis.size() == n;
    for (int k = 0; same && k < n; ++k) same = (b->psis[k] == psis[k]);
    if (!same) {
        const long long launches = b->ctx->launches;  // counted on the device, not while recording
        const int code = batch_build(b, psis);
        b->ctx->launches = launches;
        PG_TRY(code);
    }
    if (b->params_pending) PG_CUDA_TRY(cudaEventSynchronize(b->params_done));
    for (int k = 0; k < n; ++k) {
        StepParams &p = b->h_params[k];
        p.dt = dt;
        for (int q = 0; q < PG_MAX_SLOTS; ++q)
            p.h[q] = mk<double>(q < nscales ? scales[2 * ((size_t)k * nscales + q)] : 0.0,
                                q < nscales ? scales[2 * ((size_t)k * nscales + q) + 1] : 0.0);
    }
    cudaStream_t s = b->ctx->stream;
    PG_CUDA_TRY(cudaMemcpyAsync(b->d_params, b->h_params, sizeof(StepParams) * n, cudaMemcpyHostToDevice, s));
    PG_CUDA_TRY(cudaEventRecord(b->params_done, s));
    b->params_pending = true;
    PG_CUDA_TRY(cudaGraphLaunch(b->exec, s));
    return PG_OK;
}

// Per-member statistics of the last completed ensemble step (waits for the stream).
extern "C" int pg_cayley_batch_stats(pg_cayley_batch *b, pg_krylov_stats *stats)
{
    if (!b || !stats) return PG_ERR_ARG;
    PG_CUDA_TRY(cudaStreamSynchronize(b->ctx->stream));
    for (size_t k = 0; k < b->members.size(); ++k) fill_stats(b->members[k], &stats[k]);
    return PG_OK;
}
