// The m x m exponential of pAMP on the device: c = ||psi|| exp(-i dt H_k) e_1 with the
// reference's method (core/krylov/pamp/pamp/pamp.h:430-565: scaling and squaring of the
// diagonal Pade approximant of order 6, coefficients c_0 = 1, c_(i+1) = c_i (p-i)/((i+1)(2p-i)),
// N/D = I + 2 (E - O)^-1 O with the even and odd parts E, O of the numerator; the reference
// evaluates them by Horner in A^2, here from the powers A^2, A^4, A^6 - the same approximant in
// four matrix products instead of seven), run by one CTA per member. Shared by the ensemble
// graph (one kernel for all members) and the persistent ensemble kernel.
#pragma once
#include "pg_internal.cuh"

struct PampExpArgs {
    const double *cols;  // the member's Hessenberg columns (ArnoldiBuf::d_cols)
    const double *norm;  // [1] = ||psi||
    double *c;           // out: [2m] coefficients of psi = V c
    double *stats;       // out: [0] basis size used, [1] error estimate |c_(k-1)|^2 (before ||psi||), [2] 0 or -1 (singular)
    int m, double_ortho;
    double tol;
};

static __device__ __forceinline__ cxd cdiv(cxd a, cxd b)
{
    const double d = b.x * b.x + b.y * b.y;
    return mk<double>((a.x * b.x + a.y * b.y) / d, (a.y * b.x - a.x * b.y) / d);
}

// C = A B for k x k row-major matrices in shared memory (C distinct from A and B)
static __device__ void smem_matmul(int k, const cxd *A, const cxd *B, cxd *C)
{
    for (int t = threadIdx.x; t < k * k; t += blockDim.x) {
        const int i = t / k, j = t - i * k;
        cxd s = mk<double>(0.0, 0.0);
        for (int q = 0; q < k; ++q) cfma(s, A[i * k + q], B[q * k + j]);
        C[t] = s;
    }
    __syncthreads();
}

// c = ||psi|| exp(-i dt H_k) e_1 for one member's Hessenberg columns, by the CTA's threads
// (any block size that is a multiple of 32); pe_smem: 6 m^2 complex doubles, 16-byte aligned.
// Ends with every thread past a CTA barrier after its last shared-memory access.
static __device__ void pamp_expm_block(const PampExpArgs &a, double dt, unsigned char *pe_smem)
{
    const int m = a.m, tid = threadIdx.x, nt = blockDim.x;
    cxd *A = reinterpret_cast<cxd *>(pe_smem);
    cxd *A2 = A + m * m, *P = A2 + m * m, *Q = P + m * m, *T = Q + m * m, *D = T + m * m;
    __shared__ int k_sh, s_sh, piv_sh, bad_sh;
    __shared__ double red[32];
    const size_t cd = 2 * (size_t)(m + 2);
    if (tid == 0) {  // happy breakdown (pamp.h:306-313): truncate at the first small subdiagonal
        int k = m;
        for (int j = 0; j + 1 < m; ++j)
            if (a.cols[((size_t)j * 3 + 2) * cd + 2 * (j + 1) + 1] < a.tol) {
                k = j + 1;
                break;
            }
        k_sh = k;
        bad_sh = 0;
    }
    __syncthreads();
    const int k = k_sh;
    // A = -i dt H_k
    double mx = 0.0;
    for (int t = tid; t < k * k; t += nt) {
        const int i = t / k, j = t - i * k;
        cxd h = mk<double>(0.0, 0.0);
        if (i <= j) {
            const double *p0 = a.cols + ((size_t)j * 3 + 0) * cd;
            h = mk<double>(p0[2 * i], p0[2 * i + 1]);
            if (a.double_ortho) {
                const double *p1 = a.cols + ((size_t)j * 3 + 1) * cd;
                h = h + mk<double>(p1[2 * i], p1[2 * i + 1]);
            }
        } else if (i == j + 1) {
            h = mk<double>(a.cols[((size_t)j * 3 + 2) * cd + 2 * (j + 1) + 1], 0.0);
        }
        A[t] = mk<double>(dt * h.y, -dt * h.x);
        mx = fmax(mx, sqrt(A[t].x * A[t].x + A[t].y * A[t].y));
    }
    for (int o = 16; o > 0; o >>= 1) mx = fmax(mx, __shfl_xor_sync(0xffffffffu, mx, o));
    if ((tid & 31) == 0) red[tid >> 5] = mx;
    __syncthreads();
    if (tid == 0) {
        double r = 0.0;
        for (int w = 0; w < (nt + 31) / 32; ++w) r = fmax(r, red[w]);
        // a non-finite or absurdly large matrix has no useful exponential (and would ask for
        // an unbounded number of squarings): reported as singular
        if (!(r <= 1e30)) bad_sh = 1;
        s_sh = (r > 0.0 && r <= 1e30) ? max(0, (int)ceil(log2(r))) : 0;
    }
    __syncthreads();
    if (bad_sh) {
        for (int t = tid; t < 2 * m; t += nt) a.c[t] = 0.0;
        if (tid == 0) { a.stats[0] = k; a.stats[1] = 0.0; a.stats[2] = -1.0; }
        __syncthreads();
        return;
    }
    const int sq = s_sh;
    const double scale = ldexp(1.0, -sq);
    for (int t = tid; t < k * k; t += nt) A[t] = scale * A[t];
    __syncthreads();
    smem_matmul(k, A, A, A2);
    // diagonal Pade approximant of order 6: c_0 = 1, c_(i+1) = c_i (p - i) / ((i + 1)(2p - i))
    const int order = 6;
    double c[order + 1];
    c[0] = 1.0;
    for (int i = 0; i < order; ++i) c[i + 1] = c[i] * (double)(order - i) / (double)((i + 1) * (2 * order - i));
    for (int t = tid; t < k * k; t += nt) {
        const bool dg = (t / k) == (t % k);
        Q[t] = mk<double>(dg ? c[order] : 0.0, 0.0);
        P[t] = mk<double>(dg ? c[order - 1] : 0.0, 0.0);
    }
    __syncthreads();
    // even part Q = c0 + c2 B + c4 B^2 + c6 B^3 and odd part P = A (c1 + c3 B + c5 B^2) of the
    // numerator, B = A^2: four matrix products in all (B, B^2, B^3, A P')
    const bool odd = false;
    smem_matmul(k, A2, A2, T);  // B^2
    smem_matmul(k, T, A2, D);   // B^3
    for (int t = tid; t < k * k; t += nt) {
        const double dg = (t / k) == (t % k) ? 1.0 : 0.0;
        Q[t] = c[6] * D[t] + c[4] * T[t] + c[2] * A2[t] + mk<double>(c[0] * dg, 0.0);
        P[t] = c[5] * T[t] + c[3] * A2[t] + mk<double>(c[1] * dg, 0.0);
    }
    __syncthreads();
    smem_matmul(k, P, A, T);
    {
        cxd *tmp = P; P = T; T = tmp;
    }
    // solve (Q - P) X = P by LU with partial pivoting; X overwrites P
    for (int t = tid; t < k * k; t += nt) D[t] = Q[t] - P[t];
    __syncthreads();
    for (int pc = 0; pc < k; ++pc) {
        if (tid == 0) {
            int r = pc;
            double best = -1.0;
            for (int i = pc; i < k; ++i) {
                const double v = D[i * k + pc].x * D[i * k + pc].x + D[i * k + pc].y * D[i * k + pc].y;
                if (v > best) { best = v; r = i; }
            }
            piv_sh = r;
            if (best == 0.0) bad_sh = 1;
        }
        __syncthreads();
        if (bad_sh) break;
        const int r = piv_sh;
        if (r != pc)
            for (int j = tid; j < k; j += nt) {
                cxd t0 = D[pc * k + j]; D[pc * k + j] = D[r * k + j]; D[r * k + j] = t0;
                t0 = P[pc * k + j]; P[pc * k + j] = P[r * k + j]; P[r * k + j] = t0;
            }
        __syncthreads();
        for (int i = pc + 1 + tid; i < k; i += nt) D[i * k + pc] = cdiv(D[i * k + pc], D[pc * k + pc]);
        __syncthreads();
        for (int t = tid; t < (k - pc - 1) * k; t += nt) {
            const int i = pc + 1 + t / k, j = t % k;
            const cxd l = D[i * k + pc];
            if (j > pc) D[i * k + j] = D[i * k + j] - l * D[pc * k + j];
            P[i * k + j] = P[i * k + j] - l * P[pc * k + j];
        }
        __syncthreads();
    }
    if (bad_sh) {
        for (int t = tid; t < 2 * m; t += nt) a.c[t] = 0.0;
        if (tid == 0) { a.stats[0] = k; a.stats[1] = 0.0; a.stats[2] = -1.0; }
        __syncthreads();
        return;
    }
    for (int j = tid; j < k; j += nt)
        for (int i = k - 1; i >= 0; --i) {
            cxd sum = P[i * k + j];
            for (int q = i + 1; q < k; ++q) sum = sum - D[i * k + q] * P[q * k + j];
            P[i * k + j] = cdiv(sum, D[i * k + i]);
        }
    __syncthreads();
    // E = +-(I + 2 X), then squared sq times
    cxd *E = P;
    for (int t = tid; t < k * k; t += nt) {
        cxd e = 2.0 * E[t];
        if ((t / k) == (t % k)) e.x += 1.0;
        E[t] = odd ? mk<double>(-e.x, -e.y) : e;
    }
    __syncthreads();
    for (int q = 0; q < sq; ++q) {
        smem_matmul(k, E, E, T);
        for (int t = tid; t < k * k; t += nt) E[t] = T[t];
        __syncthreads();
    }
    const double nrm = a.norm[1];
    for (int i = tid; i < m; i += nt) {
        const cxd v = i < k ? E[i * k] : mk<double>(0.0, 0.0);
        a.c[2 * i] = v.x * nrm;
        a.c[2 * i + 1] = v.y * nrm;
    }
    if (tid == 0) {
        const cxd last = E[(k - 1) * k];
        a.stats[0] = k;
        a.stats[1] = last.x * last.x + last.y * last.y;
        a.stats[2] = 0.0;
    }
    __syncthreads();
}

// ---- the same exponential in double-float arithmetic -----------------------------------------
// The same method as pamp_expm_block (scaling and squaring of the diagonal Pade approximant of
// order 6 from the powers of A^2, (Q - P) X = P by LU with partial pivoting, E = I + 2X) with the
// matrices as complex double-float values (FP32 pairs hi + lo per real part, about 2^-44
// relative): the FP64 matrix products of that routine take a few hundred microseconds per
// member on one SM of this GPU. Divisions (2m^2 of them) and the final coefficients go
// through FP64.
struct dff {
    float h, l;
};
static __device__ __forceinline__ dff df_make(double x)
{
    const float h = (float)x;
    return {h, (float)(x - (double)h)};
}
static __device__ __forceinline__ double df_val(dff a) { return (double)a.h + (double)a.l; }
static __device__ __forceinline__ dff df_add(dff a, dff b)
{
    const float s = a.h + b.h;
    const float bb = s - a.h;
    const float e = ((a.h - (s - bb)) + (b.h - bb)) + (a.l + b.l);
    const float h = s + e;
    return {h, e - (h - s)};
}
// (products whose rounded value enters a two-sum are formed with __fmul_rn, which the
// compiler never contracts into an FMA with a following addition)
static __device__ __forceinline__ dff df_mul(dff a, dff b)
{
    const float p = __fmul_rn(a.h, b.h);
    const float e = fmaf(a.h, b.l, fmaf(a.l, b.h, fmaf(a.h, b.h, -p)));
    const float h = p + e;
    return {h, e - (h - p)};
}
static __device__ __forceinline__ dff df_neg(dff a) { return {-a.h, -a.l}; }
// 1 / a: the FP32 reciprocal refined by one Newton step in double-float arithmetic
static __device__ __forceinline__ dff df_recip(dff a)
{
    const dff x{1.0f / a.h, 0.f};
    const dff r = df_add({1.0f, 0.f}, df_neg(df_mul(a, x)));  // 1 - a x
    return df_add(x, df_mul(x, r));
}

typedef float4 zdf;  // (re hi, re lo, im hi, im lo)
static const int PE_DF_MAXM = 64;  // largest basis of the double-float exponential
static __device__ __forceinline__ zdf zdf_make(cxd v)
{
    const dff r = df_make(v.x), i = df_make(v.y);
    return make_float4(r.h, r.l, i.h, i.l);
}
static __device__ __forceinline__ cxd zdf_val(zdf a) { return mk<double>((double)a.x + (double)a.y, (double)a.z + (double)a.w); }
static __device__ __forceinline__ zdf zdf_add(zdf a, zdf b)
{
    const dff r = df_add({a.x, a.y}, {b.x, b.y}), i = df_add({a.z, a.w}, {b.z, b.w});
    return make_float4(r.h, r.l, i.h, i.l);
}
static __device__ __forceinline__ zdf zdf_sub(zdf a, zdf b) { return zdf_add(a, make_float4(-b.x, -b.y, -b.z, -b.w)); }
static __device__ __forceinline__ zdf zdf_mul(zdf a, zdf b)
{
    const dff ar{a.x, a.y}, ai{a.z, a.w}, br{b.x, b.y}, bi{b.z, b.w};
    const dff r = df_add(df_mul(ar, br), df_neg(df_mul(ai, bi)));
    const dff i = df_add(df_mul(ar, bi), df_mul(ai, br));
    return make_float4(r.h, r.l, i.h, i.l);
}

// 1 / d = conj(d) / |d|^2 in double-float arithmetic; false when |d|^2 is zero or not finite
static __device__ __forceinline__ bool zdf_recip(zdf d, zdf &out)
{
    const dff re{d.x, d.y}, im{d.z, d.w};
    const dff n2 = df_add(df_mul(re, re), df_mul(im, im));
    if (!(n2.h > 0.f && n2.h < 3e38f)) return false;
    const dff inv = df_recip(n2);
    const dff r = df_mul(re, inv), i = df_neg(df_mul(im, inv));
    out = make_float4(r.h, r.l, i.h, i.l);
    return true;
}

// Accumulated real product in double-float arithmetic, in the manner of the compensated dot
// product (Ogita, Rump and Oishi, "Accurate sum and dot product", SIAM J. Sci. Comput. 26,
// 2005): s + c += a b with a, b double-float; the high product split exactly by an FMA, the
// cross terms and the two-sum error gathered in c, renormalised once at the end.
struct dacc {
    float s, c;
};
static __device__ __forceinline__ void dacc_madd(dacc &u, float ah, float al, float bh, float bl)
{
    const float p = __fmul_rn(ah, bh);
    const float e = fmaf(ah, bl, fmaf(al, bh, fmaf(ah, bh, -p)));
    const float t = u.s + p;
    const float bb = t - u.s;
    u.c += ((u.s - (t - bb)) + (p - bb)) + e;
    u.s = t;
}
static __device__ __forceinline__ void dacc_merge(dacc &u, const dacc &v)
{
    const float t = u.s + v.s;
    const float bb = t - u.s;
    u.c += ((u.s - (t - bb)) + (v.s - bb)) + v.c;
    u.s = t;
}
static __device__ __forceinline__ float2 dacc_val(const dacc &u)
{
    const float h = u.s + u.c;
    return make_float2(h, u.c - (h - u.s));
}

// C = A B for k x k row-major matrices in shared memory (C distinct from A and B): each
// element's real and imaginary sums as two compensated chains over alternate terms (four
// chains in flight per thread)
static __device__ void zdf_matmul(int k, const zdf *A, const zdf *B, zdf *C)
{
    for (int t = threadIdx.x; t < k * k; t += blockDim.x) {
        const int i = t / k, j = t - i * k;
        dacc r0{0.f, 0.f}, r1{0.f, 0.f}, i0{0.f, 0.f}, i1{0.f, 0.f};
        int q = 0;
        for (; q + 1 < k; q += 2) {
            const zdf a0 = A[i * k + q], b0 = B[q * k + j];
            const zdf a1 = A[i * k + q + 1], b1 = B[(q + 1) * k + j];
            dacc_madd(r0, a0.x, a0.y, b0.x, b0.y);
            dacc_madd(r0, -a0.z, -a0.w, b0.z, b0.w);
            dacc_madd(i0, a0.x, a0.y, b0.z, b0.w);
            dacc_madd(i0, a0.z, a0.w, b0.x, b0.y);
            dacc_madd(r1, a1.x, a1.y, b1.x, b1.y);
            dacc_madd(r1, -a1.z, -a1.w, b1.z, b1.w);
            dacc_madd(i1, a1.x, a1.y, b1.z, b1.w);
            dacc_madd(i1, a1.z, a1.w, b1.x, b1.y);
        }
        if (q < k) {
            const zdf a0 = A[i * k + q], b0 = B[q * k + j];
            dacc_madd(r0, a0.x, a0.y, b0.x, b0.y);
            dacc_madd(r0, -a0.z, -a0.w, b0.z, b0.w);
            dacc_madd(i0, a0.x, a0.y, b0.z, b0.w);
            dacc_madd(i0, a0.z, a0.w, b0.x, b0.y);
        }
        dacc_merge(r0, r1);
        dacc_merge(i0, i1);
        const float2 re = dacc_val(r0), im = dacc_val(i0);
        C[t] = make_float4(re.x, re.y, im.x, im.y);
    }
    __syncthreads();
}

// c = ||psi|| exp(-i dt H_k) e_1 as pamp_expm_block computes it (same arguments and outputs)
static __device__ void pamp_expm_block_df(const PampExpArgs &a, double dt, unsigned char *pe_smem)
{
    const int m = a.m, tid = threadIdx.x, nt = blockDim.x;
    zdf *A = reinterpret_cast<zdf *>(pe_smem);
    zdf *A2 = A + m * m, *P = A2 + m * m, *Q = P + m * m, *T = Q + m * m, *D = T + m * m;
    __shared__ int k_sh, s_sh, bad_sh;
    __shared__ float red[32];
    __shared__ zdf rinv[PE_DF_MAXM];  // reciprocals of the LU pivots
    const size_t cd = 2 * (size_t)(m + 2);
    if (tid < 32) {  // happy breakdown (pamp.h:306-313): truncate at the first small subdiagonal
        int k = m;
        for (int j0 = 0; j0 + 1 < m; j0 += 32) {  // the subdiagonals loaded together, a ballot finds the first
            const int j = j0 + tid;
            const bool small = j + 1 < m && a.cols[((size_t)j * 3 + 2) * cd + 2 * (j + 1) + 1] < a.tol;
            const unsigned bal = __ballot_sync(0xffffffffu, small);
            if (bal) {
                k = j0 + __ffs(bal);
                break;
            }
        }
        if (tid == 0) {
            k_sh = k;
            bad_sh = 0;
        }
    }
    __syncthreads();
    const int k = k_sh;
    // -i dt H_k (FP64 values, double-float copies); its largest magnitude (in FP32: only its
    // power of two is used) sets the scaling
    float mx = 0.f;
    for (int t = tid; t < k * k; t += nt) {
        const int i = t / k, j = t - i * k;
        cxd h = mk<double>(0.0, 0.0);
        if (i <= j) {
            const double *p0 = a.cols + ((size_t)j * 3 + 0) * cd;
            h = mk<double>(p0[2 * i], p0[2 * i + 1]);
            if (a.double_ortho) {
                const double *p1 = a.cols + ((size_t)j * 3 + 1) * cd;
                h = h + mk<double>(p1[2 * i], p1[2 * i + 1]);
            }
        } else if (i == j + 1) {
            h = mk<double>(a.cols[((size_t)j * 3 + 2) * cd + 2 * (j + 1) + 1], 0.0);
        }
        const cxd v = mk<double>(dt * h.y, -dt * h.x);
        const float fx = (float)v.x, fy = (float)v.y;
        mx = fmaxf(mx, sqrtf(fx * fx + fy * fy));
        T[t] = zdf_make(v);  // unscaled, scaled below
    }
    for (int o = 16; o > 0; o >>= 1) mx = fmaxf(mx, __shfl_xor_sync(0xffffffffu, mx, o));
    if ((tid & 31) == 0) red[tid >> 5] = mx;
    __syncthreads();
    if (tid == 0) {
        float r = 0.f;
        for (int w = 0; w < (nt + 31) / 32; ++w) r = fmaxf(r, red[w]);
        // a non-finite or absurdly large matrix has no useful exponential (and would ask for
        // an unbounded number of squarings), nor has a basis above PE_DF_MAXM: reported as
        // singular
        if (!(r <= 1e30f) || k > PE_DF_MAXM) bad_sh = 1;
        int e = 0;
        if (r > 0.f && r <= 1e30f) {
            frexpf(r, &e);  // r = f 2^e, f in [1/2, 1): the smallest s with r 2^-s <= 1
            if (ldexpf(1.0f, e - 1) == r) e -= 1;
        }
        s_sh = max(0, e);
    }
    __syncthreads();
    if (bad_sh) {
        for (int t = tid; t < 2 * m; t += nt) a.c[t] = 0.0;
        if (tid == 0) { a.stats[0] = k; a.stats[1] = 0.0; a.stats[2] = -1.0; }
        __syncthreads();
        return;
    }
    const int sq = s_sh;
    const float scale = ldexpf(1.0f, -sq);  // a power of two: exact on both parts
    for (int t = tid; t < k * k; t += nt) {
        const zdf v = T[t];
        A[t] = make_float4(v.x * scale, v.y * scale, v.z * scale, v.w * scale);
    }
    __syncthreads();
    zdf_matmul(k, A, A, A2);
    const int order = 6;
    double c[order + 1];
    c[0] = 1.0;
    for (int i = 0; i < order; ++i) c[i + 1] = c[i] * (double)(order - i) / (double)((i + 1) * (2 * order - i));
    for (int t = tid; t < k * k; t += nt) {
        const bool dg = (t / k) == (t % k);
        Q[t] = zdf_make(mk<double>(dg ? c[order] : 0.0, 0.0));
        P[t] = zdf_make(mk<double>(dg ? c[order - 1] : 0.0, 0.0));
    }
    __syncthreads();
    // even part Q = c0 + c2 B + c4 B^2 + c6 B^3 and odd part P = A (c1 + c3 B + c5 B^2) of the
    // numerator, B = A^2: four matrix products in all (B, B^2, B^3, A P')
    const bool odd = false;
    zdf_matmul(k, A2, A2, T);  // B^2
    zdf_matmul(k, T, A2, D);   // B^3
    {
        const dff c0 = df_make(c[0]), c1 = df_make(c[1]), c2 = df_make(c[2]), c3 = df_make(c[3]), c4 = df_make(c[4]),
                  c5 = df_make(c[5]), c6 = df_make(c[6]);
        auto scl = [](dff s, zdf v) {
            const dff r = df_mul(s, {v.x, v.y}), i = df_mul(s, {v.z, v.w});
            return make_float4(r.h, r.l, i.h, i.l);
        };
        for (int t = tid; t < k * k; t += nt) {
            const bool dg = (t / k) == (t % k);
            zdf q = zdf_add(zdf_add(scl(c6, D[t]), scl(c4, T[t])), scl(c2, A2[t]));
            zdf p = zdf_add(scl(c5, T[t]), scl(c3, A2[t]));
            if (dg) {
                q = zdf_add(q, make_float4(c0.h, c0.l, 0.f, 0.f));
                p = zdf_add(p, make_float4(c1.h, c1.l, 0.f, 0.f));
            }
            Q[t] = q;
            P[t] = p;
        }
    }
    __syncthreads();
    zdf_matmul(k, P, A, T);
    {
        zdf *tmp = P; P = T; T = tmp;
    }
    for (int t = tid; t < k * k; t += nt) D[t] = zdf_sub(Q[t], P[t]);
    __syncthreads();
    // LU with partial pivoting, two CTA barriers per column: warp 0 finds the pivot (largest
    // magnitude, the first on ties; high parts in FP32), swaps the rows and forms the pivot's
    // reciprocal (double-float Newton step); then every thread eliminates its elements of the
    // rows below with its own multiplier D[i][pc] / pivot (no division per element)
    for (int pc = 0; pc < k; ++pc) {
        if (tid < 32) {
            float best = -1.f;
            int r = pc;
            for (int i = pc + tid; i < k; i += 32) {
                const zdf v = D[i * k + pc];
                const float mag = v.x * v.x + v.z * v.z;
                if (mag > best) { best = mag; r = i; }
            }
            for (int o = 16; o > 0; o >>= 1) {
                const float ob = __shfl_xor_sync(0xffffffffu, best, o);
                const int orow = __shfl_xor_sync(0xffffffffu, r, o);
                if (ob > best || (ob == best && orow < r)) { best = ob; r = orow; }
            }
            if (r != pc)
                for (int j = tid; j < k; j += 32) {
                    zdf t0 = D[pc * k + j]; D[pc * k + j] = D[r * k + j]; D[r * k + j] = t0;
                    t0 = P[pc * k + j]; P[pc * k + j] = P[r * k + j]; P[r * k + j] = t0;
                }
            __syncwarp();
            if (tid == 0) {
                zdf r;
                if (zdf_recip(D[pc * k + pc], r)) rinv[pc] = r;
                else bad_sh = 1;
            }
        }
        __syncthreads();
        if (bad_sh) break;
        const zdf rp = rinv[pc];
        for (int t = tid; t < (k - pc - 1) * k; t += nt) {
            const int i = pc + 1 + t / k, j = t % k;
            const zdf l = zdf_mul(D[i * k + pc], rp);
            if (j > pc) D[i * k + j] = zdf_sub(D[i * k + j], zdf_mul(l, D[pc * k + j]));
            P[i * k + j] = zdf_sub(P[i * k + j], zdf_mul(l, P[pc * k + j]));
        }
        __syncthreads();
    }
    if (bad_sh) {
        for (int t = tid; t < 2 * m; t += nt) a.c[t] = 0.0;
        if (tid == 0) { a.stats[0] = k; a.stats[1] = 0.0; a.stats[2] = -1.0; }
        __syncthreads();
        return;
    }
    // back substitution, one warp per column of X: row i's sum over q > i by the lanes (a
    // compensated product each, merged by shuffles in a fixed order), then lane 0 forms X[i][j]
    const int lane = tid & 31, warp = tid >> 5, nw = nt >> 5;
    for (int j = warp; j < k; j += nw) {
        for (int i = k - 1; i >= 0; --i) {
            dacc sr{0.f, 0.f}, si{0.f, 0.f};
            for (int q = i + 1 + lane; q < k; q += 32) {
                const zdf d = D[i * k + q], x = P[q * k + j];
                dacc_madd(sr, d.x, d.y, x.x, x.y);
                dacc_madd(sr, -d.z, -d.w, x.z, x.w);
                dacc_madd(si, d.x, d.y, x.z, x.w);
                dacc_madd(si, d.z, d.w, x.x, x.y);
            }
#pragma unroll
            for (int o = 16; o > 0; o >>= 1) {
                const dacc orr{__shfl_xor_sync(0xffffffffu, sr.s, o), __shfl_xor_sync(0xffffffffu, sr.c, o)};
                const dacc oi{__shfl_xor_sync(0xffffffffu, si.s, o), __shfl_xor_sync(0xffffffffu, si.c, o)};
                dacc_merge(sr, orr);
                dacc_merge(si, oi);
            }
            if (lane == 0) {
                const float2 r = dacc_val(sr), im = dacc_val(si);
                P[i * k + j] = zdf_mul(zdf_sub(P[i * k + j], make_float4(r.x, r.y, im.x, im.y)), rinv[i]);
            }
            __syncwarp();
        }
    }
    __syncthreads();
    zdf *E = P;  // +-(I + 2 X), then squared sq times
    for (int t = tid; t < k * k; t += nt) {
        zdf e = E[t];
        e = make_float4(2.f * e.x, 2.f * e.y, 2.f * e.z, 2.f * e.w);
        if ((t / k) == (t % k)) e = zdf_add(e, make_float4(1.f, 0.f, 0.f, 0.f));
        E[t] = odd ? make_float4(-e.x, -e.y, -e.z, -e.w) : e;
    }
    __syncthreads();
    // all but the last rs squarings as matrix products (ping-pong between E and T); the first
    // column of E^(2^rs) then by 2^rs - 1 products of E with its first column (one warp per
    // row, compensated sums merged by shuffles)
    const int rs = min(sq, 4);
    zdf *F = T;
    for (int q = 0; q < sq - rs; ++q) {
        zdf_matmul(k, E, E, F);
        zdf *tmp = E; E = F; F = tmp;
    }
    zdf *v = F, *w = F + k;  // F is free: two vectors of k
    for (int i = tid; i < k; i += nt) v[i] = E[i * k];
    __syncthreads();
    for (int it = 0; it < (1 << rs) - 1; ++it) {
        for (int i = warp; i < k; i += nw) {
            dacc sr{0.f, 0.f}, si{0.f, 0.f};
            for (int q = lane; q < k; q += 32) {
                const zdf e = E[i * k + q], x = v[q];
                dacc_madd(sr, e.x, e.y, x.x, x.y);
                dacc_madd(sr, -e.z, -e.w, x.z, x.w);
                dacc_madd(si, e.x, e.y, x.z, x.w);
                dacc_madd(si, e.z, e.w, x.x, x.y);
            }
#pragma unroll
            for (int o = 16; o > 0; o >>= 1) {
                const dacc orr{__shfl_xor_sync(0xffffffffu, sr.s, o), __shfl_xor_sync(0xffffffffu, sr.c, o)};
                const dacc oi{__shfl_xor_sync(0xffffffffu, si.s, o), __shfl_xor_sync(0xffffffffu, si.c, o)};
                dacc_merge(sr, orr);
                dacc_merge(si, oi);
            }
            if (lane == 0) {
                const float2 r = dacc_val(sr), im = dacc_val(si);
                w[i] = make_float4(r.x, r.y, im.x, im.y);
            }
        }
        __syncthreads();
        zdf *tmp = v; v = w; w = tmp;
    }
    const double nrm = a.norm[1];
    for (int i = tid; i < m; i += nt) {
        const cxd val = i < k ? zdf_val(v[i]) : mk<double>(0.0, 0.0);
        a.c[2 * i] = val.x * nrm;
        a.c[2 * i + 1] = val.y * nrm;
    }
    if (tid == 0) {
        const cxd last = zdf_val(v[k - 1]);
        a.stats[0] = k;
        a.stats[1] = last.x * last.x + last.y * last.y;
        a.stats[2] = 0.0;
    }
    __syncthreads();
}
