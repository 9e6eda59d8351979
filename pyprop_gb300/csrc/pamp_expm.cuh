// The m x m exponential of pAMP on the device: c = ||psi|| exp(-i dt H_k) e_1 with the
// reference's method (core/krylov/pamp/pamp/pamp.h:430-565: scaling and squaring of the
// diagonal Pade approximant of order 6, coefficients c_0 = 1, c_(i+1) = c_i (p-i)/((i+1)(2p-i)),
// Horner in A^2, N/D = I + 2 (E - O)^-1 O), run by one CTA per member. Shared by the ensemble
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
        s_sh = r > 0.0 ? max(0, (int)ceil(log2(r))) : 0;
    }
    __syncthreads();
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
    bool odd = true;
    for (int i = order - 2; i >= 0; --i) {
        cxd *M = odd ? Q : P;
        smem_matmul(k, M, A2, T);
        for (int t = tid; t < k * k; t += nt) M[t] = T[t] + mk<double>((t / k) == (t % k) ? c[i] : 0.0, 0.0);
        __syncthreads();
        odd = !odd;
    }
    {
        cxd *M = odd ? Q : P;
        smem_matmul(k, M, A, T);
        for (int t = tid; t < k * k; t += nt) M[t] = T[t];
        __syncthreads();
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
