// Factorized rank-3 terms: V = sum_q w_q s_slot(q) A_q (x) R_q.
//
// The two-electron repulsion in coupled spherical harmonics is, per angular pair, a sum over
// multipoles l3 of an angular coefficient times the radial function r<^l3 / r>^(l3+1)
// (examples/tensor/helium_stabilization/coupledspherical.cpp:7-127). The reference
// represents the sum per angular pair on SelectionRule_R12 x banded-packed x
// banded-nonhermitian; here each multipole's radial operator R_q is stored once (a band x
// band block on the two radial ranks, real) and the angular coefficients A_q as a sparse
// matrix, so the term costs one radial block per multipole instead of one per angular pair.
//
// One application, after the banded part of the operator has written dst:
//   mix:    Z[q][a'] = w_q s_slot(q) sum_a A_q[a'][a] src[a]       (per point of the N1 x N2 grid)
//   radial: dst[a'][i1][i2] += sum_q sum_{d1,d2} R_q[i1][d1][d2][i2] Z[q][a'][i1+d1-k][i2+d2-k]
// The mix handles the factors in chunks of QC (accumulators in registers, src re-read per
// chunk from L1/L2); rows without entries in a chunk skip it, and their scratch rows stay at
// the zeros written at upload. The radial kernel is a 169-point stencil (k = 6) with
// coefficients varying per point and shared by all channels: a CTA stages one radial row of
// Z for CA channels (transposed, channels innermost) and the matching row of R in shared
// memory, and each thread keeps PI consecutive points x PC channels of accumulators and a
// sliding window of PI rows of Z in registers, so each shared-memory load feeds 4 PC (or PI x
// PC / 2 for the window) fused multiply-adds. It is bound by FP32 (or FP64) FMA throughput.
#include "pg_internal.cuh"

#include <algorithm>
#include <cmath>
#include <map>

namespace {

const int QC = 16;  // factors per register chunk of the mix kernel

struct FactArgs {
    int Q, Qp, A, N1, N2, N2p, nct;
    const int *row_ptr, *col, *qlo, *qhi, *slot;
    const void *coef;
    const unsigned char *chunk, *bflag;
    const void *radial;
    const cxd *w;
    void *Z;
};

FactArgs args_of(const FactDev &f)
{
    FactArgs a;
    a.Q = f.Q; a.Qp = f.Qp; a.A = f.A; a.N1 = f.N1; a.N2 = f.N2; a.N2p = f.N2p; a.nct = f.nct;
    a.row_ptr = f.row_ptr; a.col = f.col; a.qlo = f.qlo; a.qhi = f.qhi; a.slot = f.slot;
    a.coef = f.coef; a.chunk = f.chunk; a.bflag = f.bflag; a.radial = f.radial; a.w = f.w; a.Z = f.Z;
    return a;
}

// Z[q][a][p] = w_q s_slot(q) / inv_scale * sum_e coef[e][q] x[col_e][p]; one CTA = 128 points
// of one output row a.
template <typename R>
__global__ void __launch_bounds__(128) fact_mix_kernel(FactArgs f, pg_scales scales, const cxd *__restrict__ scales_dev,
                                                       const cx<R> *__restrict__ x, const double *__restrict__ inv_scale)
{
    const int a = blockIdx.y;
    const long long NP = (long long)f.N1 * f.N2;
    const long long p = (long long)blockIdx.x * 128 + threadIdx.x;
    const bool live = p < NP;
    const double sc = inv_scale ? 1.0 / *inv_scale : 1.0;
    const int e0 = f.row_ptr[a], e1 = f.row_ptr[a + 1];
    const int nch = f.Qp / QC;
    const R *__restrict__ coef = (const R *)f.coef;
    cx<R> *__restrict__ Z = (cx<R> *)f.Z;
    for (int k = 0; k < nch; ++k) {
        if (!f.chunk[(size_t)a * nch + k]) continue;
        const int q0 = k * QC;
        cx<R> acc[QC];
#pragma unroll
        for (int j = 0; j < QC; ++j) acc[j] = mk<R>((R)0, (R)0);
        for (int e = e0; e < e1; ++e) {
            if (f.qhi[e] < q0 || f.qlo[e] >= q0 + QC) continue;
            const cx<R> xv = live ? x[(size_t)f.col[e] * NP + p] : mk<R>((R)0, (R)0);
            const R *__restrict__ c = coef + (size_t)e * f.Qp + q0;
#pragma unroll
            for (int j = 0; j < QC; ++j) {
                const R cj = c[j];
                acc[j].x = fma(cj, xv.x, acc[j].x);
                acc[j].y = fma(cj, xv.y, acc[j].y);
            }
        }
        if (!live) continue;
#pragma unroll
        for (int j = 0; j < QC; ++j) {
            const int q = q0 + j;
            if (q >= f.Q) break;
            const cxd s = scales_dev ? scales_dev[f.slot[q]] : scales.s[f.slot[q]];
            const cxd ws = sc * (f.w[q] * s);
            Z[((size_t)q * f.A + a) * NP + p] = cvt<R>(ws) * acc[j];
        }
    }
}

// PC consecutive complex values from 16-byte aligned shared memory
template <typename R, int PC>
__device__ __forceinline__ void load_row(const cx<R> *p, cx<R> (&out)[PC])
{
    if constexpr (sizeof(R) == 4) {
        static_assert(PC % 2 == 0, "float rows load in pairs");
#pragma unroll
        for (int h = 0; h < PC / 2; ++h) {
            const float4 v = reinterpret_cast<const float4 *>(p)[h];
            out[2 * h] = mk<R>(v.x, v.y);
            out[2 * h + 1] = mk<R>(v.z, v.w);
        }
    } else {
#pragma unroll
        for (int h = 0; h < PC; ++h) out[h] = p[h];
    }
}

template <typename R, int PI>
__device__ __forceinline__ void load_coefs(const R *p, R (&out)[PI])
{
    if constexpr (sizeof(R) == 4) {
        static_assert(PI % 4 == 0, "float coefficients load in fours");
#pragma unroll
        for (int h = 0; h < PI / 4; ++h) {
            const float4 v = reinterpret_cast<const float4 *>(p)[h];
            out[4 * h] = v.x; out[4 * h + 1] = v.y; out[4 * h + 2] = v.z; out[4 * h + 3] = v.w;
        }
    } else {
        static_assert(PI % 2 == 0, "double coefficients load in pairs");
#pragma unroll
        for (int h = 0; h < PI / 2; ++h) {
            const double2 v = reinterpret_cast<const double2 *>(p)[h];
            out[2 * h] = v.x; out[2 * h + 1] = v.y;
        }
    }
}

// Shared-memory position (in complex elements) of window row j, channel c. Rows are CA + 2
// complex long (a multiple of 16 bytes); every other block of PI rows is shifted by 16 bytes so
// that the four point groups of a warp, which read rows PI apart, fall on different banks.
template <typename R, int CA, int PI>
__device__ __forceinline__ int zpos(int j, int c)
{
    constexpr int OFF = 16 / (int)sizeof(cx<R>);
    return j * (CA + 2) + ((j / PI) & 1) * OFF + c;
}

// One CTA = radial row i1 (blockIdx.x), T2 points of the last rank (blockIdx.y), CA channels
// (blockIdx.z); thread = PI consecutive points x PC channels.
template <typename R, int KB, int T2, int CA, int PI, int PC>
__global__ void __launch_bounds__((T2 / PI) * (CA / PC), 2)
    fact_radial_kernel(FactArgs f, cx<R> *__restrict__ y)
{
    constexpr int B = 2 * KB + 1;
    constexpr int TW = T2 + 2 * KB;
    constexpr int NT = (T2 / PI) * (CA / PC);
    constexpr int TCN = CA / PC;
    constexpr int ZELEMS = TW * (CA + 2) + 16 / (int)sizeof(cx<R>);
    extern __shared__ __align__(16) unsigned char smem_raw[];
    cx<R> *zs = reinterpret_cast<cx<R> *>(smem_raw);
    R *rs = reinterpret_cast<R *>(smem_raw + (size_t)ZELEMS * sizeof(cx<R>));

    const int i1 = blockIdx.x, t0 = blockIdx.y * T2, c0 = blockIdx.z * CA;
    const int tid = threadIdx.x;
    const int tc = tid % TCN, ti = tid / TCN;
    const int N1 = f.N1, N2 = f.N2, A = f.A;
    const long long NP = (long long)N1 * N2;
    const cx<R> *__restrict__ Z = (const cx<R> *)f.Z;
    const R *__restrict__ radial = (const R *)f.radial;

    cx<R> acc[PI][PC];
#pragma unroll
    for (int p = 0; p < PI; ++p)
#pragma unroll
        for (int c = 0; c < PC; ++c) acc[p][c] = mk<R>((R)0, (R)0);

    for (int q = 0; q < f.Q; ++q) {
        if (!f.bflag[(size_t)q * f.nct + blockIdx.z]) continue;
        for (int d1 = 0; d1 < B; ++d1) {
            const int j1 = i1 + d1 - KB;
            if (j1 < 0 || j1 >= N1) continue;
            const R *__restrict__ Rrow = radial + (((size_t)q * N1 + i1) * B + d1) * B * (size_t)f.N2p;
            __syncthreads();  // the previous stage's reads are done
            for (int idx = tid; idx < CA * TW; idx += NT) {
                const int c = idx / TW, j = idx - c * TW;
                const int ch = c0 + c, j2 = t0 - KB + j;
                cx<R> v = mk<R>((R)0, (R)0);
                if (ch < A && j2 >= 0 && j2 < N2) v = Z[((size_t)q * A + ch) * NP + (size_t)j1 * N2 + j2];
                zs[zpos<R, CA, PI>(j, c)] = v;
            }
            for (int idx = tid; idx < B * T2; idx += NT) {
                const int d2 = idx / T2, i = idx - d2 * T2;
                const int i2 = t0 + i;
                rs[idx] = i2 < N2 ? Rrow[(size_t)d2 * f.N2p + i2] : (R)0;
            }
            __syncthreads();
            cx<R> win[PI + B - 1][PC];
#pragma unroll
            for (int r = 0; r < PI - 1; ++r) load_row<R, PC>(zs + zpos<R, CA, PI>(ti * PI + r, tc * PC), win[r]);
#pragma unroll
            for (int d2 = 0; d2 < B; ++d2) {
                load_row<R, PC>(zs + zpos<R, CA, PI>(ti * PI + d2 + PI - 1, tc * PC), win[d2 + PI - 1]);
                R rv[PI];
                load_coefs<R, PI>(rs + d2 * T2 + ti * PI, rv);
#pragma unroll
                for (int p = 0; p < PI; ++p)
#pragma unroll
                    for (int c = 0; c < PC; ++c) {
                        acc[p][c].x = fma(rv[p], win[p + d2][c].x, acc[p][c].x);
                        acc[p][c].y = fma(rv[p], win[p + d2][c].y, acc[p][c].y);
                    }
            }
        }
    }
#pragma unroll
    for (int c = 0; c < PC; ++c) {
        const int ch = c0 + tc * PC + c;
        if (ch >= A) continue;
        cx<R> *__restrict__ yr = y + (size_t)ch * NP + (size_t)i1 * N2;
#pragma unroll
        for (int p = 0; p < PI; ++p) {
            const int i2 = t0 + ti * PI + p;
            if (i2 < N2) yr[i2] = yr[i2] + acc[p][c];
        }
    }
}

// tile shapes per precision
template <typename R> struct RadialTile;
template <> struct RadialTile<float> { static const int T2 = 128, CA = 32, PI = 8, PC = 4; };
template <> struct RadialTile<double> { static const int T2 = 64, CA = 16, PI = 4, PC = 2; };

template <typename R>
size_t radial_smem(int kb)
{
    typedef RadialTile<R> T;
    const int TW = T::T2 + 2 * kb;
    const size_t z = ((size_t)TW * (T::CA + 2) + 16 / sizeof(cx<R>)) * sizeof(cx<R>);
    return z + (size_t)(2 * kb + 1) * T::T2 * sizeof(R);
}

template <typename R>
int launch_factored(pg_op *op, const pg_scales &scales, const cxd *scales_dev, const void *src, void *dst,
                    const double *inv_scale)
{
    typedef RadialTile<R> T;
    const FactDev &fd = op->fact;
    const FactArgs fa = args_of(fd);
    cudaStream_t s = op->ctx->stream;
    const long long NP = (long long)fd.N1 * fd.N2;
    dim3 g1((unsigned)((NP + 127) / 128), (unsigned)fd.A);
    fact_mix_kernel<R><<<g1, 128, 0, s>>>(fa, scales, scales_dev, (const cx<R> *)src, inv_scale);
    op->ctx->launches++;
    PG_TRY(pg_check_launch(op->ctx));
    dim3 g2((unsigned)fd.N1, (unsigned)((fd.N2 + T::T2 - 1) / T::T2), (unsigned)fd.nct);
    const int nt = (T::T2 / T::PI) * (T::CA / T::PC);
    const size_t sm = radial_smem<R>(op->kb);
    switch (op->kb) {
    case 6:
        fact_radial_kernel<R, 6, T::T2, T::CA, T::PI, T::PC><<<g2, nt, sm, s>>>(fa, (cx<R> *)dst);
        break;
    default: return PG_ERR_STORAGE;
    }
    op->ctx->launches++;
    return pg_check_launch(op->ctx);
}

}  // namespace

int pg_factored_apply(pg_op *op, const pg_scales &scales, const cxd *scales_dev, const void *src, void *dst,
                      const double *src_inv_scale_dev)
{
    if (op->fact.Q == 0) return PG_OK;
    return op->precision == PG_FP64 ? launch_factored<double>(op, scales, scales_dev, src, dst, src_inv_scale_dev)
                                    : launch_factored<float>(op, scales, scales_dev, src, dst, src_inv_scale_dev);
}

void pg_factored_free(pg_op *op)
{
    FactDev &f = op->fact;
    cudaFree(f.row_ptr); cudaFree(f.col); cudaFree(f.qlo); cudaFree(f.qhi); cudaFree(f.slot);
    cudaFree(f.coef); cudaFree(f.chunk); cudaFree(f.bflag); cudaFree(f.radial); cudaFree(f.w); cudaFree(f.Z);
    f = FactDev();
}

extern "C" int pg_op_add_factored(pg_op *op, int nfactors, const double *radial, const double *weights,
                                  const int *slots, long long nentries, const int *ent_factor, const int *ent_row,
                                  const int *ent_col, const double *ent_coef)
{
    if (!op || nfactors < 0 || nentries < 0) return PG_ERR_ARG;
    if (op->finalized) return PG_ERR_STATE;
    if (op->rank != 3) return PG_ERR_STORAGE;
    if (nfactors == 0) return PG_OK;
    if (!radial || !weights || !slots || (nentries > 0 && (!ent_factor || !ent_row || !ent_col || !ent_coef)))
        return PG_ERR_ARG;
    if (op->kb != 6) return PG_ERR_STORAGE;  // the radial stencil is compiled for 13 diagonals
    const int A = op->shape[0], N1 = op->shape[1], N2 = op->shape[2], b = op->b;
    if (N1 <= 2 * op->kb) return PG_ERR_SHAPE;
    if (op->factors.size() + nfactors > (size_t)4096) return PG_ERR_ARG;
    for (int q = 0; q < nfactors; ++q)
        if (slots[q] < 0 || slots[q] >= PG_MAX_SLOTS) return PG_ERR_ARG;
    for (long long e = 0; e < nentries; ++e)
        if (ent_factor[e] < 0 || ent_factor[e] >= nfactors || ent_row[e] < 0 || ent_row[e] >= A || ent_col[e] < 0 ||
            ent_col[e] >= A)
            return PG_ERR_SHAPE;
    const size_t rsz = (size_t)N1 * b * b * N2;
    const size_t first = op->factors.size();
    for (int q = 0; q < nfactors; ++q) {
        HostFactor h;
        h.radial.assign(radial + rsz * q, radial + rsz * (q + 1));
        h.w[0] = weights[2 * q];
        h.w[1] = weights[2 * q + 1];
        h.slot = slots[q];
        op->factors.push_back(std::move(h));
    }
    for (long long e = 0; e < nentries; ++e) {
        HostFactor &h = op->factors[first + ent_factor[e]];
        h.row.push_back(ent_row[e]);
        h.col.push_back(ent_col[e]);
        h.coef.push_back(ent_coef[e]);
    }
    return PG_OK;
}

template <typename R>
static int upload_real(void **dst, const std::vector<double> &src)
{
    std::vector<R> tmp(src.size());
    for (size_t k = 0; k < src.size(); ++k) tmp[k] = (R)src[k];
    PG_CUDA_TRY(cudaMalloc(dst, std::max<size_t>(1, tmp.size()) * sizeof(R)));
    if (!tmp.empty()) PG_CUDA_TRY(cudaMemcpy(*dst, tmp.data(), tmp.size() * sizeof(R), cudaMemcpyHostToDevice));
    return PG_OK;
}

template <typename T>
static int upload_vec(T **dst, const std::vector<T> &src)
{
    PG_CUDA_TRY(cudaMalloc((void **)dst, std::max<size_t>(1, src.size()) * sizeof(T)));
    if (!src.empty()) PG_CUDA_TRY(cudaMemcpy(*dst, src.data(), src.size() * sizeof(T), cudaMemcpyHostToDevice));
    return PG_OK;
}

int pg_factored_finalize(pg_op *op)
{
    if (op->factors.empty()) return PG_OK;
    FactDev &f = op->fact;
    const int A = op->shape[0], N1 = op->shape[1], N2 = op->shape[2], b = op->b, kb = op->kb;
    const bool fp64 = op->precision == PG_FP64;
    const int Q = (int)op->factors.size();
    f.A = A; f.N1 = N1; f.N2 = N2; f.Q = Q;
    f.Qp = (Q + QC - 1) / QC * QC;
    f.N2p = (N2 + 3) & ~3;
    const int CA = fp64 ? RadialTile<double>::CA : RadialTile<float>::CA;
    f.nct = (A + CA - 1) / CA;
    // angular rows: coefficient vector over the factors per (row, col)
    std::vector<std::map<int, std::vector<double>>> rows(A);
    for (int q = 0; q < Q; ++q) {
        const HostFactor &h = op->factors[q];
        for (size_t e = 0; e < h.row.size(); ++e) {
            std::vector<double> &v = rows[h.row[e]][h.col[e]];
            if (v.empty()) v.assign(f.Qp, 0.0);
            v[q] += h.coef[e];
        }
    }
    const int nch = f.Qp / QC;
    std::vector<int> row_ptr(A + 1, 0), col, qlo, qhi;
    std::vector<double> coef;
    std::vector<unsigned char> chunk((size_t)A * nch, 0), bflag((size_t)Q * f.nct, 0);
    std::vector<long long> rows_of_q(Q, 0);
    double mix_terms = 0;
    for (int a = 0; a < A; ++a) {
        std::vector<unsigned char> row_has(Q, 0);
        for (const auto &kv : rows[a]) {
            int lo = f.Qp, hi = -1;
            for (int q = 0; q < Q; ++q)
                if (kv.second[q] != 0.0) {
                    lo = std::min(lo, q);
                    hi = std::max(hi, q);
                    row_has[q] = 1;
                }
            if (hi < 0) continue;  // all coefficients zero
            col.push_back(kv.first);
            qlo.push_back(lo);
            qhi.push_back(hi);
            coef.insert(coef.end(), kv.second.begin(), kv.second.end());
            for (int k = lo / QC; k <= hi / QC; ++k) {
                chunk[(size_t)a * nch + k] = 1;
                mix_terms += QC;
            }
        }
        row_ptr[a + 1] = (int)col.size();
        for (int q = 0; q < Q; ++q)
            if (row_has[q]) {
                bflag[(size_t)q * f.nct + a / CA] = 1;
                rows_of_q[q]++;
            }
    }
    f.nE = (int)col.size();
    // radial factors, last rank padded to N2p; points outside the grid are dropped
    std::vector<double> rad((size_t)Q * N1 * b * b * f.N2p, 0.0);
    double pts = 0;  // in-grid stencil points of one factor
    for (int i1 = 0; i1 < N1; ++i1)
        for (int d1 = 0; d1 < b; ++d1) {
            const int j1 = i1 + d1 - kb;
            if (j1 < 0 || j1 >= N1) continue;
            for (int i2 = 0; i2 < N2; ++i2)
                for (int d2 = 0; d2 < b; ++d2) {
                    const int j2 = i2 + d2 - kb;
                    if (j2 >= 0 && j2 < N2) pts += 1;
                }
        }
    double radial_terms = 0;
    for (int q = 0; q < Q; ++q) {
        const std::vector<double> &h = op->factors[q].radial;
        for (int i1 = 0; i1 < N1; ++i1)
            for (int d1 = 0; d1 < b; ++d1)
                for (int d2 = 0; d2 < b; ++d2)
                    for (int i2 = 0; i2 < N2; ++i2) {
                        const int j1 = i1 + d1 - kb, j2 = i2 + d2 - kb;
                        if (j1 < 0 || j1 >= N1 || j2 < 0 || j2 >= N2) continue;
                        rad[(((size_t)q * N1 + i1) * b + d1) * b * f.N2p + (size_t)d2 * f.N2p + i2] =
                            h[(((size_t)i1 * b + d1) * b + d2) * N2 + i2];
                    }
        radial_terms += pts * (double)rows_of_q[q];
    }
    const double NP = (double)N1 * N2;
    f.flops_mix = 4.0 * mix_terms * NP;      // complex x real = 2 FMA per factor, entry and point
    f.flops_radial = 4.0 * radial_terms;     // per in-grid stencil point and nonzero row
    const size_t esz = fp64 ? sizeof(double) : sizeof(float);
    f.radial_bytes = (double)rad.size() * esz;
    f.z_bytes = (double)Q * A * NP * 2 * esz;
    std::vector<double> w(2 * (size_t)Q);
    std::vector<int> slot(Q);
    for (int q = 0; q < Q; ++q) {
        w[2 * q] = op->factors[q].w[0];
        w[2 * q + 1] = op->factors[q].w[1];
        slot[q] = op->factors[q].slot;
    }
    PG_TRY(upload_vec(&f.row_ptr, row_ptr));
    PG_TRY(upload_vec(&f.col, col));
    PG_TRY(upload_vec(&f.qlo, qlo));
    PG_TRY(upload_vec(&f.qhi, qhi));
    PG_TRY(upload_vec(&f.slot, slot));
    PG_TRY(upload_vec(&f.chunk, chunk));
    PG_TRY(upload_vec(&f.bflag, bflag));
    PG_CUDA_TRY(cudaMalloc(&f.w, sizeof(cxd) * Q));
    PG_CUDA_TRY(cudaMemcpy(f.w, w.data(), sizeof(cxd) * Q, cudaMemcpyHostToDevice));
    PG_TRY(fp64 ? upload_real<double>(&f.coef, coef) : upload_real<float>(&f.coef, coef));
    PG_TRY(fp64 ? upload_real<double>(&f.radial, rad) : upload_real<float>(&f.radial, rad));
    const size_t zbytes = (size_t)Q * A * (size_t)N1 * N2 * 2 * esz;
    PG_CUDA_TRY(cudaMalloc(&f.Z, zbytes));
    PG_CUDA_TRY(cudaMemset(f.Z, 0, zbytes));  // rows without entries are read as zeros
    const size_t sm = fp64 ? radial_smem<double>(kb) : radial_smem<float>(kb);
    if (fp64)
        PG_CUDA_TRY(cudaFuncSetAttribute(fact_radial_kernel<double, 6, 64, 16, 4, 2>,
                                         cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm));
    else
        PG_CUDA_TRY(cudaFuncSetAttribute(fact_radial_kernel<float, 6, 128, 32, 8, 4>,
                                         cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm));
    return PG_OK;
}

extern "C" int pg_op_factored_info(const pg_op *op, double *info)
{
    if (!op || !info) return PG_ERR_ARG;
    const FactDev &f = op->fact;
    info[0] = f.Q;
    info[1] = f.nE;
    info[2] = f.flops_mix;
    info[3] = f.flops_radial;
    info[4] = f.radial_bytes;
    info[5] = f.z_bytes;
    return PG_OK;
}
