// Adjoint of the fused density path: given cotangents of rho and grad rho on a
// grid, the gradients of a loss with respect to the MO coefficients, the primitive
// exponents and contraction coefficients, and the nuclear coordinates.  AO tiles
// are recomputed, never stored.
//
// Forward being differentiated (orbkit/core.py:266-300 with the AO kernel of
// orbkit/c_grid-based.c:9-79):
//   chi_k = g_k P_k(X,Y,Z) sum_p w_p e^{-alpha_p r^2},  w_p = c_p N(alpha_p),
//   phi_i = sum_k C_ik chi_k,  rho = sum_i o_i phi_i^2,  d_d rho = 2 sum_i o_i phi_i d_d phi_i.
// With cotangents gr (rho) and gd (d = x, y, z) per point:
//   W_i = 2 o_i (gr phi_i + sum_d gd d_d phi_i) = dL/dphi_i,   V_i = 2 o_i phi_i,
//   dL/dC_ik   = sum_r W_i chi_k + V_i G_k,          G_k = sum_d gd d_d chi_k,
//   A_k = sum_i C_ik W_i,  B_k = sum_i C_ik V_i      (AO-level cotangents),
//   dL/dalpha_p = sum_r (w'_p - w_p r^2) e_p (S0 + S1 - 2 alpha_p S2) - 2 w_p e_p S2,
//   dL/dc_p     = sum_r N_p e_p (S0 + S1 - 2 alpha_p S2),
//     S0 = sum_k A_k g_k P_k,  S1 = sum_k B_k g_k Q_k,  S2 = sum_k B_k g_k T_k,
//     Q_k = sum_d gd dP_k/dX_d,  T_k = sum_d gd X_d P_k,
//   dL/dR_A,u  = -sum_r sum_{k on A} A_k d_u chi_k + B_k sum_d gd d_u d_d chi_k   (exact second derivatives).
//
// Tile: 32 points x 8 warps.  Phase 1 (per chunk of shells): AO value + gradient
// in shared memory, MO value + gradient accumulated per warp (6 MOs each) -> W, V
// in shared memory; with more than 48 MOs, phase 1 runs once per block of 48 MOs
// and W, V go to the CTA's slot of the workspace.  Phase 2 (per chunk again): AO value, gradient and all second
// derivatives; A, B, G per (column, point); the dC pairs; per shell the exponent,
// coefficient and nuclear terms, reduced over the warp's 32 points.  Partial sums
// go to per-CTA slots of the caller's workspace (no atomics) and a second kernel
// adds the slots in a fixed order, so results are deterministic.
#include "okg_internal.cuh"

namespace okg {
namespace adj {

constexpr int P = 32;
constexpr int NW = 8;
constexpr int NT = P * NW;
constexpr int MB = 6;
constexpr int NMOMAX = NW * MB;
constexpr int KC = OKG_KC;
// Persistent CTAs: two per SM in FP32 (at most 128 registers per thread, 72 KB of
// shared memory each), one in FP64.
template <typename T>
__host__ __device__ constexpr int ctas_per_sm() { return sizeof(T) == 4 ? 2 : 1; }

template <typename T>
struct Args {
    int nmo;
    const double* C;       // nmo x ncart
    const double* occ;     // nmo
    const double* g_rho;   // npts (ld)
    const double* g_grad;  // 3 x ld, or null
    long long ld;
    T* part_c;  // [nblk][nmo][ncart]
    T* part_p;  // [nblk][nprim][2]
    T* part_g;  // [nblk][NW][natom][3]
    T* part_w;  // nmo > NMOMAX: [nblk][2][nmo][P] (W and V of the CTA's tile), else null
    long long ntiles;
};

template <typename T>
__device__ __forceinline__ T expT(T x);
template <>
__device__ __forceinline__ double expT<double>(double x) { return exp(x); }
template <>
__device__ __forceinline__ float expT<float>(float x) { return expf(x); }

template <typename T>
__device__ __forceinline__ Radial<T> radialT(const BasisDev& B, const Shell& sh, T rr, bool n1, bool n2)
{
    Radial<T> r{T(0), T(0), T(0)};
    for (int q = 0; q < sh.nprim; ++q) {
        const T a = (T)B.prim[2 * (sh.prim0 + q)];
        const T w = (T)B.prim[2 * (sh.prim0 + q) + 1];
        const T e = w * expT<T>(-a * rr);
        r.R0 += e;
        if (n1) r.R1 += a * e;
        if (n2) r.R2 += a * a * e;
    }
    return r;
}

template <typename T>
__device__ __forceinline__ T warp_sum(T v)
{
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    return v;
}

// S0, S1, S2 of one shell at one point (canonical components, compile-time powers)
template <int L, typename T>
__device__ __forceinline__ void shell_sums(T X, T Y, T Z, T gx, T gy, T gz, const BasisDev& B, const Shell& sh,
                                           const T* A_s, const T* B_s, int rowbase, int lane, T& S0, T& S1, T& S2)
{
    T px[L + 2], py[L + 2], pz[L + 2];
    px[0] = py[0] = pz[0] = T(1);
#pragma unroll
    for (int i = 1; i < L + 2; ++i) {
        px[i] = px[i - 1] * X;
        py[i] = py[i - 1] * Y;
        pz[i] = pz[i - 1] * Z;
    }
    [&]<int... J>(std::integer_sequence<int, J...>) {
        (
            [&] {
                constexpr int a = canon_l(L, J, 0), b = canon_l(L, J, 1), c = canon_l(L, J, 2);
                const int row = B.comp_row[sh.comp0 + J];
                if (row < 0) return;
                const T g = (T)B.comp_g[sh.comp0 + J];
                const T Ak = A_s[(rowbase + row) * P + lane] * g;
                const T Bk = B_s[(rowbase + row) * P + lane] * g;
                const T Pk = px[a] * py[b] * pz[c];
                T Qk = T(0);
                if (a > 0) Qk += gx * T(a) * px[a > 0 ? a - 1 : 0] * py[b] * pz[c];
                if (b > 0) Qk += gy * T(b) * px[a] * py[b > 0 ? b - 1 : 0] * pz[c];
                if (c > 0) Qk += gz * T(c) * px[a] * py[b] * pz[c > 0 ? c - 1 : 0];
                const T Tk = gx * px[a + 1] * py[b] * pz[c] + gy * px[a] * py[b + 1] * pz[c] + gz * px[a] * py[b] * pz[c + 1];
                S0 += Ak * Pk;
                S1 += Bk * Qk;
                S2 += Bk * Tk;
            }(),
            ...);
    }(std::make_integer_sequence<int, ncanon(L)>{});
}

template <typename T>
__device__ __forceinline__ void shell_sums_L(int L, T X, T Y, T Z, T gx, T gy, T gz, const BasisDev& B,
                                             const Shell& sh, const T* A_s, const T* B_s, int rowbase, int lane,
                                             T& S0, T& S1, T& S2)
{
    switch (L) {
    case 0: shell_sums<0>(X, Y, Z, gx, gy, gz, B, sh, A_s, B_s, rowbase, lane, S0, S1, S2); break;
    case 1: shell_sums<1>(X, Y, Z, gx, gy, gz, B, sh, A_s, B_s, rowbase, lane, S0, S1, S2); break;
    case 2: shell_sums<2>(X, Y, Z, gx, gy, gz, B, sh, A_s, B_s, rowbase, lane, S0, S1, S2); break;
    case 3: shell_sums<3>(X, Y, Z, gx, gy, gz, B, sh, A_s, B_s, rowbase, lane, S0, S1, S2); break;
    default: shell_sums<4>(X, Y, Z, gx, gy, gz, B, sh, A_s, B_s, rowbase, lane, S0, S1, S2); break;
    }
}

template <typename T, bool BIG>
__global__ void __launch_bounds__(NT, ctas_per_sm<T>()) adjoint_kernel(BasisDev B, Grid g, Args<T> A)
{
    extern __shared__ __align__(16) unsigned char sm_raw[];
    T* AO_s = (T*)sm_raw;            // 10 x KC x P
    T* C_s = AO_s + 10 * KC * P;     // NMOMAX x KC
    T* W_s = C_s + NMOMAX * KC;      // NMOMAX x P
    T* V_s = W_s + NMOMAX * P;       // NMOMAX x P
    T* A_s = V_s + NMOMAX * P;       // KC x P
    T* B_s = A_s + KC * P;           // KC x P
    T* G_s = B_s + KC * P;           // KC x P
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    const long long blk = blockIdx.x;
    // up to NMOMAX MOs: W, V and the coefficient chunks in shared memory; more MOs:
    // W, V in the CTA's slot of the workspace and the coefficients read from global
    // memory, the MOs of phase 1 formed in blocks of NMOMAX (AO tiles recomputed
    // per block)
    T* Wv;
    T* Vv;
    if constexpr (BIG) {
        Wv = A.part_w + blk * 2ll * A.nmo * P;
        Vv = Wv + (long long)A.nmo * P;
    } else {
        Wv = W_s;
        Vv = V_s;
    }
    T* pc = A.part_c + blk * (long long)A.nmo * B.ncart;
    T* pp = A.part_p + blk * 2ll * B.nprim;
    T* pg = A.part_g + blk * (long long)NW * B.natom * 3;
    for (long long i = tid; i < (long long)A.nmo * B.ncart; i += NT) pc[i] = T(0);
    for (long long i = tid; i < 2ll * B.nprim; i += NT) pp[i] = T(0);
    for (long long i = tid; i < (long long)NW * B.natom * 3; i += NT) pg[i] = T(0);
    __syncthreads();

    for (long long tile = blockIdx.x; tile < A.ntiles; tile += gridDim.x) {
        const long long p = tile * P + lane;
        const bool valid = p < g.npts;
        double xd, yd, zd;
        grid_point(g, valid ? p : g.npts - 1, xd, yd, zd);
        // cotangents; zero for padding points so that they contribute nothing
        const T gr = valid ? (T)A.g_rho[p] : T(0);
        const T gx = (valid && A.g_grad) ? (T)A.g_grad[p] : T(0);
        const T gy = (valid && A.g_grad) ? (T)A.g_grad[A.ld + p] : T(0);
        const T gz = (valid && A.g_grad) ? (T)A.g_grad[2 * A.ld + p] : T(0);

        // ---------------- phase 1: MOs and their gradients (blocks of NMOMAX MOs)
        for (int mb0 = 0; mb0 < A.nmo; mb0 += NMOMAX) {
        T acc[MB][4];
#pragma unroll
        for (int m = 0; m < MB; ++m)
#pragma unroll
            for (int c = 0; c < 4; ++c) acc[m][c] = T(0);
        for (int ci = 0; ci < B.nchunk; ++ci) {
            const int4 ck = B.chunks[ci];
            const int kc = ck.w - ck.z;
            __syncthreads();
            for (int i = tid; i < NMOMAX * KC; i += NT) {
                const int m = i / KC, kk = i % KC;
                C_s[i] = (mb0 + m < A.nmo && kk < kc) ? (T)A.C[(long long)(mb0 + m) * B.ncart + ck.z + kk] : T(0);
            }
            for (int s = ck.x + warp; s < ck.y; s += NW) {
                const Shell sh = B.shells[s];
                const T X = (T)(xd - B.atoms[4 * sh.atom]);
                const T Y = (T)(yd - B.atoms[4 * sh.atom + 1]);
                const T Z = (T)(zd - B.atoms[4 * sh.atom + 2]);
                const T rr = (T)((xd - B.atoms[4 * sh.atom]) * (xd - B.atoms[4 * sh.atom]) +
                                 (yd - B.atoms[4 * sh.atom + 1]) * (yd - B.atoms[4 * sh.atom + 1]) +
                                 (zd - B.atoms[4 * sh.atom + 2]) * (zd - B.atoms[4 * sh.atom + 2]));
                const Radial<T> r = radialT<T>(B, sh, rr, true, false);
                const int rowbase = sh.cart0 - ck.z;
                shell_eval_L(sh.L, X, Y, Z, r, 0xFu, false, [&](int ch, int j, T v) {
                    const int row = B.comp_row[sh.comp0 + j];
                    if (row < 0) return;
                    AO_s[(ch * KC + rowbase + row) * P + lane] = v * (T)B.comp_g[sh.comp0 + j];
                });
            }
            __syncthreads();
            for (int kk = 0; kk < kc; ++kk) {
                T a[4];
#pragma unroll
                for (int c = 0; c < 4; ++c) a[c] = AO_s[(c * KC + kk) * P + lane];
#pragma unroll
                for (int m = 0; m < MB; ++m) {
                    const T cm = C_s[(warp * MB + m) * KC + kk];
#pragma unroll
                    for (int c = 0; c < 4; ++c) acc[m][c] += cm * a[c];
                }
            }
        }
#pragma unroll
        for (int m = 0; m < MB; ++m) {
            const int mo = mb0 + warp * MB + m;
            T w = T(0), v = T(0);
            if (mo < A.nmo) {
                const T o2 = T(2) * (T)A.occ[mo];
                w = o2 * (gr * acc[m][0] + gx * acc[m][1] + gy * acc[m][2] + gz * acc[m][3]);
                v = o2 * acc[m][0];
            }
            if (mo < A.nmo || !BIG) {
                Wv[mo * P + lane] = w;
                Vv[mo * P + lane] = v;
            }
        }
        }

        // ---------------- phase 2: gradients
        for (int ci = 0; ci < B.nchunk; ++ci) {
            const int4 ck = B.chunks[ci];
            const int kc = ck.w - ck.z;
            __syncthreads();
            if constexpr (!BIG)
                for (int i = tid; i < NMOMAX * KC; i += NT) {
                    const int m = i / KC, kk = i % KC;
                    C_s[i] = (m < A.nmo && kk < kc) ? (T)A.C[(long long)m * B.ncart + ck.z + kk] : T(0);
                }
            for (int s = ck.x + warp; s < ck.y; s += NW) {
                const Shell sh = B.shells[s];
                const T X = (T)(xd - B.atoms[4 * sh.atom]);
                const T Y = (T)(yd - B.atoms[4 * sh.atom + 1]);
                const T Z = (T)(zd - B.atoms[4 * sh.atom + 2]);
                const T rr = (T)((xd - B.atoms[4 * sh.atom]) * (xd - B.atoms[4 * sh.atom]) +
                                 (yd - B.atoms[4 * sh.atom + 1]) * (yd - B.atoms[4 * sh.atom + 1]) +
                                 (zd - B.atoms[4 * sh.atom + 2]) * (zd - B.atoms[4 * sh.atom + 2]));
                const Radial<T> r = radialT<T>(B, sh, rr, true, true);
                const int rowbase = sh.cart0 - ck.z;
                shell_eval_L(sh.L, X, Y, Z, r, 0x3FFu, false, [&](int ch, int j, T v) {
                    const int row = B.comp_row[sh.comp0 + j];
                    if (row < 0) return;
                    AO_s[(ch * KC + rowbase + row) * P + lane] = v * (T)B.comp_g[sh.comp0 + j];
                });
            }
            __syncthreads();
            for (int kk = warp; kk < kc; kk += NW) {
                T a = T(0), b = T(0);
                for (int i = 0; i < A.nmo; ++i) {
                    T c;
                    if constexpr (BIG)
                        c = (T)__ldg(A.C + (long long)i * B.ncart + ck.z + kk);
                    else
                        c = C_s[i * KC + kk];
                    a += c * Wv[i * P + lane];
                    b += c * Vv[i * P + lane];
                }
                A_s[kk * P + lane] = a;
                B_s[kk * P + lane] = b;
                G_s[kk * P + lane] = gx * AO_s[(1 * KC + kk) * P + lane] + gy * AO_s[(2 * KC + kk) * P + lane] +
                                     gz * AO_s[(3 * KC + kk) * P + lane];
            }
            __syncthreads();
            // dL/dC pairs (i, column); the point loop starts at a per-thread offset
            // so that the threads of a warp read different banks
            for (int q = tid; q < A.nmo * kc; q += NT) {
                const int i = q / kc, kk = q % kc;
                T sacc = T(0);
                for (int t = 0; t < P; ++t) {
                    const int pt = (t + lane) & (P - 1);
                    sacc += Wv[i * P + pt] * AO_s[kk * P + pt] + Vv[i * P + pt] * G_s[kk * P + pt];
                }
                pc[(long long)i * B.ncart + ck.z + kk] += sacc;
            }
            // exponents, contraction coefficients, nuclear coordinates
            for (int s = ck.x + warp; s < ck.y; s += NW) {
                const Shell sh = B.shells[s];
                const double Xd = xd - B.atoms[4 * sh.atom], Yd = yd - B.atoms[4 * sh.atom + 1],
                             Zd = zd - B.atoms[4 * sh.atom + 2];
                const T X = (T)Xd, Y = (T)Yd, Z = (T)Zd;
                const T rr = (T)(Xd * Xd + Yd * Yd + Zd * Zd);
                const int rowbase = sh.cart0 - ck.z;
                T S0 = T(0), S1 = T(0), S2 = T(0);
                shell_sums_L(sh.L, X, Y, Z, gx, gy, gz, B, sh, A_s, B_s, rowbase, lane, S0, S1, S2);
                T rx = T(0), ry = T(0), rz = T(0);
                for (int row = 0; row < sh.ncart; ++row) {
                    const int k = rowbase + row;
                    const T Ak = A_s[k * P + lane], Bk = B_s[k * P + lane];
                    const T cx = AO_s[(1 * KC + k) * P + lane], cy = AO_s[(2 * KC + k) * P + lane],
                            cz = AO_s[(3 * KC + k) * P + lane];
                    const T cxx = AO_s[(4 * KC + k) * P + lane], cyy = AO_s[(5 * KC + k) * P + lane],
                            czz = AO_s[(6 * KC + k) * P + lane], cxy = AO_s[(7 * KC + k) * P + lane],
                            cxz = AO_s[(8 * KC + k) * P + lane], cyz = AO_s[(9 * KC + k) * P + lane];
                    rx += Ak * cx + Bk * (gx * cxx + gy * cxy + gz * cxz);
                    ry += Ak * cy + Bk * (gx * cxy + gy * cyy + gz * cyz);
                    rz += Ak * cz + Bk * (gx * cxz + gy * cyz + gz * czz);
                }
                rx = warp_sum(rx);
                ry = warp_sum(ry);
                rz = warp_sum(rz);
                if (lane == 0) {
                    T* gslot = pg + ((long long)warp * B.natom + sh.atom) * 3;
                    gslot[0] -= rx;
                    gslot[1] -= ry;
                    gslot[2] -= rz;
                }
                const T F = S0 + S1;
                for (int q = 0; q < sh.nprim; ++q) {
                    const int pi = sh.prim0 + q;
                    const T a = (T)B.prim[2 * pi], w = (T)B.prim[2 * pi + 1];
                    const T dw = (T)B.prim_adj[2 * pi], nrm = (T)B.prim_adj[2 * pi + 1];
                    const T e = expT<T>(-a * rr);
                    const T Fa = F - T(2) * a * S2;
                    T da = (dw - w * rr) * e * Fa - T(2) * w * e * S2;
                    T dc = nrm * e * Fa;
                    da = warp_sum(da);
                    dc = warp_sum(dc);
                    if (lane == 0) {
                        pp[2 * pi] += da;
                        pp[2 * pi + 1] += dc;
                    }
                }
            }
        }
    }
}

template <typename T>
__global__ void reduce_kernel(const T* __restrict__ part, long long n, int nblk, int inner, double* __restrict__ out)
{
    // out[j] = sum over blocks b (and `inner` consecutive sub-slots) of part[b][.][j], fixed order
    long long j = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    if (j >= n) return;
    double s = 0.0;
    for (int b = 0; b < nblk; ++b)
        for (int w = 0; w < inner; ++w) s += (double)part[((long long)b * inner + w) * n + j];
    out[j] = s;
}

template <typename T>
size_t workspace_bytes(const okg_basis* b, int nmo, int nblk)
{
    const size_t wv = nmo > NMOMAX ? 2 * (size_t)nmo * P : 0;  // W and V of the CTA's tile
    return (size_t)nblk * ((size_t)nmo * b->ncart + 2 * (size_t)b->nprim + (size_t)NW * b->natom * 3 + wv) * sizeof(T) +
           256;
}

template <typename T>
static int block_count(long long ntiles)
{
    int dev = 0, sms = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    if (sms <= 0) sms = 1;
    const long long cap = (long long)sms * ctas_per_sm<T>();
    return (int)(ntiles < cap ? (ntiles > 0 ? ntiles : 1) : cap);
}

template <typename T>
static int run(const okg_basis* b, const Grid& g, int nmo, const double* C, const double* occ, const double* grho,
               const double* ggrad, long long ld, double* dC, double* dprim, double* dgeo, void* work,
               size_t work_bytes, cudaStream_t st)
{
    const long long ntiles = (g.npts + P - 1) / P;
    const int nblk = block_count<T>(ntiles);
    if (work_bytes < workspace_bytes<T>(b, nmo, nblk))
        return set_error(OKG_ERR_ARG, "okg_rho_backward: workspace smaller than okg_rho_backward_workspace reports");
    Args<T> A;
    A.nmo = nmo;
    A.C = C;
    A.occ = occ;
    A.g_rho = grho;
    A.g_grad = ggrad;
    A.ld = ld;
    A.part_c = (T*)work;
    A.part_p = A.part_c + (size_t)nblk * nmo * b->ncart;
    A.part_g = A.part_p + (size_t)nblk * 2 * b->nprim;
    A.part_w = nmo > NMOMAX ? A.part_g + (size_t)nblk * NW * b->natom * 3 : nullptr;
    A.ntiles = ntiles;
    const size_t smem = sizeof(T) * (10 * KC * P + NMOMAX * KC + 2 * NMOMAX * P + 3 * KC * P);
    static bool configured = false;
    if (!configured) {
        cudaError_t e =
            cudaFuncSetAttribute(adjoint_kernel<T, false>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
        if (e == cudaSuccess)
            e = cudaFuncSetAttribute(adjoint_kernel<T, true>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
        if (e != cudaSuccess) return cuda_status(e, "okg_rho_backward: smem attribute");
        configured = true;
    }
    if (nmo > NMOMAX)
        adjoint_kernel<T, true><<<nblk, NT, smem, st>>>(b->dev, g, A);
    else
        adjoint_kernel<T, false><<<nblk, NT, smem, st>>>(b->dev, g, A);
    long long n = (long long)nmo * b->ncart;
    reduce_kernel<T><<<(unsigned)((n + 255) / 256), 256, 0, st>>>(A.part_c, n, nblk, 1, dC);
    n = 2ll * b->nprim;
    reduce_kernel<T><<<(unsigned)((n + 255) / 256), 256, 0, st>>>(A.part_p, n, nblk, 1, dprim);
    n = 3ll * b->natom;
    reduce_kernel<T><<<(unsigned)((n + 255) / 256), 256, 0, st>>>(A.part_g, n, nblk, NW, dgeo);
    return cuda_status(cudaGetLastError(), "okg_rho_backward launch");
}

}  // namespace adj
}  // namespace okg

using namespace okg;

extern "C" int okg_rho_backward_workspace(const okg_basis* b, const okg_grid* grid, int nmo, int precision,
                                          size_t* bytes)
{
    if (!b || !grid || !bytes || nmo <= 0) return set_error(OKG_ERR_ARG, "okg_rho_backward_workspace: bad argument");
    const long long ntiles = (grid->npts + adj::P - 1) / adj::P;
    *bytes = precision == 32 ? adj::workspace_bytes<float>(b, nmo, adj::block_count<float>(ntiles))
                             : adj::workspace_bytes<double>(b, nmo, adj::block_count<double>(ntiles));
    return OKG_OK;
}

extern "C" int okg_rho_backward(const okg_basis* b, const okg_grid* gr, int nmo, const double* d_coeff,
                                const double* d_occ, const double* d_g_rho, const double* d_g_grad, int64_t ld,
                                int precision, double* d_dcoeff, double* d_dprim, double* d_dgeo, void* d_work,
                                size_t work_bytes, okg_stream stream)
{
    if (!b || !gr || !d_coeff || !d_occ || !d_g_rho || !d_dcoeff || !d_dprim || !d_dgeo || !d_work || nmo <= 0)
        return set_error(OKG_ERR_ARG, "okg_rho_backward: NULL argument or nmo <= 0");
    if (precision != 32 && precision != 64) return set_error(OKG_ERR_ARG, "okg_rho_backward: precision 32 or 64");
    Grid g;
    g.x = gr->d_x;
    g.y = gr->d_y;
    g.z = gr->d_z;
    g.npts = gr->npts;
    g.offset = gr->offset;
    g.nx = gr->nx;
    g.ny = gr->ny;
    g.nz = gr->nz;
    g.regular = gr->regular;
    if (g.npts <= 0 || !g.x || !g.y || !g.z) return set_error(OKG_ERR_ARG, "okg_rho_backward: bad grid");
    if (g.regular && (g.nx <= 0 || g.ny <= 0 || g.nz <= 0 || g.offset < 0 ||
                      g.offset + g.npts > (long long)g.nx * g.ny * g.nz))
        return set_error(OKG_ERR_ARG, "okg_rho_backward: regular grid range outside Nx*Ny*Nz");
    if (ld < g.npts) return set_error(OKG_ERR_ARG, "okg_rho_backward: ld < npts");
    cudaStream_t st = (cudaStream_t)stream;
    if (precision == 64)
        return adj::run<double>(b, g, nmo, d_coeff, d_occ, d_g_rho, d_g_grad, ld, d_dcoeff, d_dprim, d_dgeo, d_work,
                                work_bytes, st);
    return adj::run<float>(b, g, nmo, d_coeff, d_occ, d_g_rho, d_g_grad, ld, d_dcoeff, d_dprim, d_dgeo, d_work,
                           work_bytes, st);
}
