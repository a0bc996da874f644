// Learned orbit surrogate for sm_103a: training data from the FP64 integrator, a fused BF16
// tensor-core training step (mma.sync m16n8k16, FP32 accumulation), Adam, the views' tables built
// on the fifth-generation tensor cores (tcgen05, tc_mlp.cuh), and the surrogate trace with its
// fallback list.
//
// Network (3 -> 64 -> 64 -> 64 -> 2, SiLU): inputs x1 = scaled log r_cam, x2 = scaled
// sign(beta) ln(1 + |beta|/eps) with beta = b / sqrt(27) - 1, x3 = orbit coordinate sigma
// (surrogate_math.cuh); outputs y = (polar angle of the integrated orbit - closed-form baseline)
// / y_scale at sigma, and a capture logit. The first layer runs in FP32 on the CUDA cores, the
// two 64x64 layers in BF16 on the tensor cores, every activation rounded to BF16, identically in
// training and inference. SiLU uses the SFU tanh: silu(z) = h + h tanh(h) with h = z/2. The output
// layer is FP32 in training; in inference it runs on the tensor cores with W4 split into three
// BF16 parts (FP32 accuracy).
//
// Fragment layout (PTX ISA, mma.m16n8k16 .bf16): with g = lane / 4, t = lane % 4, a thread holds
// A rows g and g+8, columns 2t, 2t+1, 2t+8, 2t+9; B column g, rows 2t, 2t+1, 2t+8, 2t+9; C rows
// g and g+8, columns 2t, 2t+1. A layer's C tiles (n = 8j..8j+7) therefore become the next layer's
// A tiles (k = 16i..16i+15) from tiles 2i and 2i+1 without leaving registers.
#include <cuda_bf16.h>
#include <cuda_runtime.h>

#include <algorithm>

#include "surrogate.cuh"
#include "surrogate_math.cuh"
#include "tc_mlp.cuh"

namespace bhr {
namespace surr {

namespace {

constexpr float kSqrt27f = 5.19615242270663f;
constexpr double kSqrt27d = 5.196152422706632;

// ---------------------------------------------------------------------------------------
// small helpers
__device__ __forceinline__ float tanh_sfu(float x) {
    float y;
    asm("tanh.approx.f32 %0, %1;" : "=f"(y) : "f"(x));
    return y;
}
// d silu / dz = s + z s (1 - s), s = 1/2 + tanh(z/2)/2
__device__ __forceinline__ float silu_grad(float z) {
    const float s = fmaf(0.5f, tanh_sfu(0.5f * z), 0.5f);
    return fmaf(z * s, 1.0f - s, s);
}
__device__ __forceinline__ uint32_t pack_bf16(float lo, float hi) {
    __nv_bfloat162 v = __floats2bfloat162_rn(lo, hi);
    return *reinterpret_cast<uint32_t*>(&v);
}
__device__ __forceinline__ uint32_t lds32(const __nv_bfloat16* p) { return *reinterpret_cast<const uint32_t*>(p); }
// one 32-byte store (p 32-byte aligned)
__device__ __forceinline__ void st_global_v8(const void* p, uint32_t a, uint32_t b, uint32_t c, uint32_t d, uint32_t e,
                                             uint32_t f, uint32_t g, uint32_t h) {
    asm volatile("st.global.v8.b32 [%0], {%1, %2, %3, %4, %5, %6, %7, %8};" ::"l"(p), "r"(a), "r"(b), "r"(c), "r"(d),
                 "r"(e), "r"(f), "r"(g), "r"(h)
                 : "memory");
}
__device__ __forceinline__ uint32_t pack2(__nv_bfloat16 lo, __nv_bfloat16 hi) {
    return uint32_t(__bfloat16_as_ushort(lo)) | (uint32_t(__bfloat16_as_ushort(hi)) << 16);
}
// silu of two half pre-activations h = z/2, fma(h, tanh h, h) in FP32, rounded to a BF16 pair (lo
// in bits 0-15): a BF16 A-fragment register as it stands. (The packed tanh.approx.bf16x2 /
// fma.rn.bf16x2 form measured 0.8% slower on the surrogate pass: the SFU spends the same time on
// a packed pair as on two scalars, and the network is noisier.)
__device__ __forceinline__ uint32_t silu_pair_h(float lo, float hi) {
    return pack_bf16(fmaf(lo, tanh_sfu(lo), lo), fmaf(hi, tanh_sfu(hi), hi));
}
__device__ __forceinline__ float bf_lo(uint32_t v) { return __uint_as_float(v << 16); }
__device__ __forceinline__ float bf_hi(uint32_t v) { return __uint_as_float(v & 0xffff0000u); }
__device__ __forceinline__ void mma_bf16(float (&c)[4], const uint32_t (&a)[4], uint32_t b0, uint32_t b1) {
    asm volatile(
        "mma.sync.aligned.m16n8k16.row.col.f32.bf16.bf16.f32 {%0,%1,%2,%3}, {%4,%5,%6,%7}, {%8,%9}, "
        "{%0,%1,%2,%3};"
        : "+f"(c[0]), "+f"(c[1]), "+f"(c[2]), "+f"(c[3])
        : "r"(a[0]), "r"(a[1]), "r"(a[2]), "r"(a[3]), "r"(b0), "r"(b1));
}

// Network weights in shared memory.
struct SmemNet {
    __nv_bfloat16 w2[kH * kLd];  // [out][in]
    __nv_bfloat16 w3[kH * kLd];
    // inference only: the output layer as one n = 8 tile of BF16 B operands, [n][k]: rows 0-1 the
    // BF16 parts of W4's two rows, rows 2-3 the BF16 parts of the remainders, rows 4-5 the rest
    // (hi + mid + lo = W4 to 24 bits), rows 6-7 zero
    __nv_bfloat16 w4s[8 * kLd];
    float4 w1[kH];               // {w[f][0], w[f][1], w[f][2], b[f]}
    float b2[kH], b3[kH];
    float w4[kOut * kH];
    float b4[kOut];
};
// Transposed hidden weights for the backward pass: wT[in][out].
struct SmemNetT {
    __nv_bfloat16 w2t[kH * kLd];
    __nv_bfloat16 w3t[kH * kLd];
};

__device__ void load_net(SmemNet& N, SmemNetT* T, const float* __restrict__ P) {
    for (int k = threadIdx.x; k < kH * kH; k += blockDim.x) {
        const int o = k / kH, i = k % kH;
        const __nv_bfloat16 a = __float2bfloat16_rn(P[kW2 + k]);
        const __nv_bfloat16 c = __float2bfloat16_rn(P[kW3 + k]);
        N.w2[o * kLd + i] = a;
        N.w3[o * kLd + i] = c;
        if (T) {
            T->w2t[i * kLd + o] = a;
            T->w3t[i * kLd + o] = c;
        }
    }
    for (int f = threadIdx.x; f < kH; f += blockDim.x) {
        N.w1[f] = make_float4(P[kW1 + 3 * f], P[kW1 + 3 * f + 1], P[kW1 + 3 * f + 2], P[kB1 + f]);
        N.b2[f] = P[kB2 + f];
        N.b3[f] = P[kB3 + f];
        N.w4[f] = P[kW4 + f];
        N.w4[kH + f] = P[kW4 + kH + f];
    }
    if (threadIdx.x < kOut) N.b4[threadIdx.x] = P[kB4 + threadIdx.x];
}

__device__ __forceinline__ void st_pair(__nv_bfloat16* p, uint32_t v) { *reinterpret_cast<uint32_t*>(p) = v; }

// Layer 1 (FP32) for rows ra, rb of a 16-row tile: pre-activations z and BF16 A fragments of
// silu(z) for the 16 features f = 16i + 2t + {0, 1, 8, 9} this thread owns.
template <bool kStore>
__device__ __forceinline__ void layer1(const SmemNet& N, const float4& xa, const float4& xb, uint32_t (&A)[4][4],
                                       int t, __nv_bfloat16* zs, __nv_bfloat16* hs, int ra, int rb) {
#pragma unroll
    for (int i = 0; i < 4; ++i) {
        float za[4], zb[4];
#pragma unroll
        for (int q = 0; q < 4; ++q) {
            const int f = 16 * i + 2 * t + (q & 1) + ((q & 2) ? 8 : 0);
            const float4 w = N.w1[f];
            za[q] = fmaf(w.x, xa.x, fmaf(w.y, xa.y, fmaf(w.z, xa.z, w.w)));
            zb[q] = fmaf(w.x, xb.x, fmaf(w.y, xb.y, fmaf(w.z, xb.z, w.w)));
            if (kStore) {
                zs[ra * kLd + f] = __float2bfloat16_rn(za[q]);
                zs[rb * kLd + f] = __float2bfloat16_rn(zb[q]);
            }
        }
        A[i][0] = silu_pair_h(0.5f * za[0], 0.5f * za[1]);
        A[i][1] = silu_pair_h(0.5f * zb[0], 0.5f * zb[1]);
        A[i][2] = silu_pair_h(0.5f * za[2], 0.5f * za[3]);
        A[i][3] = silu_pair_h(0.5f * zb[2], 0.5f * zb[3]);
        if (kStore) {
            const int f = 16 * i + 2 * t;
            st_pair(&hs[ra * kLd + f], A[i][0]);
            st_pair(&hs[rb * kLd + f], A[i][1]);
            st_pair(&hs[ra * kLd + f + 8], A[i][2]);
            st_pair(&hs[rb * kLd + f + 8], A[i][3]);
        }
    }
}

// C = A W^T + bias for a 64x64 BF16 layer (W in shared memory, [n][k] with row stride kLd).
__device__ __forceinline__ void mma_layer(const __nv_bfloat16* W, const float* bias, const uint32_t (&A)[4][4],
                                          float (&C)[8][4], int g, int t) {
#pragma unroll
    for (int j = 0; j < 8; ++j) {
        const float c0 = bias ? bias[8 * j + 2 * t] : 0.f;
        const float c1 = bias ? bias[8 * j + 2 * t + 1] : 0.f;
        C[j][0] = c0;
        C[j][1] = c1;
        C[j][2] = c0;
        C[j][3] = c1;
#pragma unroll
        for (int i = 0; i < 4; ++i) {
            const __nv_bfloat16* wp = W + (8 * j + g) * kLd + 16 * i + 2 * t;
            mma_bf16(C[j], A[i], lds32(wp), lds32(wp + 8));
        }
    }
}

// C tiles (FP32 pre-activations z) -> silu -> next layer's A fragments (BF16).
__device__ __forceinline__ void act_pack(const float (&C)[8][4], uint32_t (&A)[4][4]) {
#pragma unroll
    for (int i = 0; i < 4; ++i) {
        A[i][0] = silu_pair_h(0.5f * C[2 * i][0], 0.5f * C[2 * i][1]);
        A[i][1] = silu_pair_h(0.5f * C[2 * i][2], 0.5f * C[2 * i][3]);
        A[i][2] = silu_pair_h(0.5f * C[2 * i + 1][0], 0.5f * C[2 * i + 1][1]);
        A[i][3] = silu_pair_h(0.5f * C[2 * i + 1][2], 0.5f * C[2 * i + 1][3]);
    }
}

// C tiles (FP32, no activation) -> BF16 A fragments (used for gradients dz).
__device__ __forceinline__ void pack_only(const float (&C)[8][4], uint32_t (&A)[4][4]) {
#pragma unroll
    for (int i = 0; i < 4; ++i) {
        A[i][0] = pack_bf16(C[2 * i][0], C[2 * i][1]);
        A[i][1] = pack_bf16(C[2 * i][2], C[2 * i][3]);
        A[i][2] = pack_bf16(C[2 * i + 1][0], C[2 * i + 1][1]);
        A[i][3] = pack_bf16(C[2 * i + 1][2], C[2 * i + 1][3]);
    }
}

// Output layer (FP32) on z3 tiles: o[row][out] for rows g and g+8, reduced over the quad.
__device__ __forceinline__ void out_layer(const SmemNet& N, const float (&Z)[8][4], float (&o)[2][2], int t) {
    float pa0 = 0.f, pa1 = 0.f, pb0 = 0.f, pb1 = 0.f;
#pragma unroll
    for (int j = 0; j < 8; ++j) {
        const int f = 8 * j + 2 * t;
        const uint32_t sa = silu_pair_h(0.5f * Z[j][0], 0.5f * Z[j][1]), sb = silu_pair_h(0.5f * Z[j][2], 0.5f * Z[j][3]);
        const float h00 = bf_lo(sa), h01 = bf_hi(sa), h10 = bf_lo(sb), h11 = bf_hi(sb);
        const float w0a = N.w4[f], w0b = N.w4[f + 1], w1a = N.w4[kH + f], w1b = N.w4[kH + f + 1];
        pa0 = fmaf(w0a, h00, fmaf(w0b, h01, pa0));
        pa1 = fmaf(w1a, h00, fmaf(w1b, h01, pa1));
        pb0 = fmaf(w0a, h10, fmaf(w0b, h11, pb0));
        pb1 = fmaf(w1a, h10, fmaf(w1b, h11, pb1));
    }
#pragma unroll
    for (int m = 1; m <= 2; m <<= 1) {
        pa0 += __shfl_xor_sync(0xffffffffu, pa0, m);
        pa1 += __shfl_xor_sync(0xffffffffu, pa1, m);
        pb0 += __shfl_xor_sync(0xffffffffu, pb0, m);
        pb1 += __shfl_xor_sync(0xffffffffu, pb1, m);
    }
    o[0][0] = pa0 + N.b4[0];
    o[0][1] = pa1 + N.b4[1];
    o[1][0] = pb0 + N.b4[0];
    o[1][1] = pb1 + N.b4[1];
}

// ---------------------------------------------------------------------------------------
// training data: FP64 RK4 in the orbital plane (x'' = -3 h^2 x / r^5, the reference's equation)

__device__ __forceinline__ uint64_t splitmix(uint64_t x) {
    x += 0x9E3779B97F4A7C15ull;
    x = (x ^ (x >> 30)) * 0xBF58476D1CE4E5B9ull;
    x = (x ^ (x >> 27)) * 0x94D049BB133111EBull;
    return x ^ (x >> 31);
}
__device__ __forceinline__ double unif(uint64_t& s) {
    s = splitmix(s);
    return double(s >> 11) * (1.0 / 9007199254740992.0);
}

struct P2 {
    double x, y;
};
__device__ __forceinline__ P2 acc2(P2 p, double m3h2) {
    const double r2 = p.x * p.x + p.y * p.y;
    const double ri = rsqrt(r2);
    const double k = m3h2 * ri * ri * ri * ri * ri;
    return {k * p.x, k * p.y};
}

// Polar angle at which the cubic Hermite arc between (x0, m0) and (x1, m1) reaches radius R,
// relative to x0 (m = v dt). Newton on |p(tau)|^2 = R^2 from linear interpolation of r.
__device__ double hermite_angle(P2 x0, P2 m0, P2 x1, P2 m1, double r0, double r1, double R) {
    double tau = (R - r0) / (r1 - r0);
    tau = tau < 0.0 ? 0.0 : (tau > 1.0 ? 1.0 : tau);
    P2 p{0, 0};
    for (int it = 0; it < 6; ++it) {
        const double t2 = tau * tau, t3 = t2 * tau;
        const double h00 = 2 * t3 - 3 * t2 + 1, h10 = t3 - 2 * t2 + tau, h01 = -2 * t3 + 3 * t2, h11 = t3 - t2;
        const double d00 = 6 * t2 - 6 * tau, d10 = 3 * t2 - 4 * tau + 1, d01 = -6 * t2 + 6 * tau, d11 = 3 * t2 - 2 * tau;
        p = {h00 * x0.x + h10 * m0.x + h01 * x1.x + h11 * m1.x, h00 * x0.y + h10 * m0.y + h01 * x1.y + h11 * m1.y};
        const P2 dp{d00 * x0.x + d10 * m0.x + d01 * x1.x + d11 * m1.x, d00 * x0.y + d10 * m0.y + d01 * x1.y + d11 * m1.y};
        const double f = p.x * p.x + p.y * p.y - R * R;
        const double df = 2 * (p.x * dp.x + p.y * dp.y);
        if (df == 0.0) break;
        tau -= f / df;
        tau = tau < 0.0 ? 0.0 : (tau > 1.0 ? 1.0 : tau);
    }
    return atan2(x0.x * p.y - x0.y * p.x, x0.x * p.x + x0.y * p.y);
}

constexpr int kMaxK = 8;

__global__ void __launch_bounds__(128) k_orbit_data(uint64_t seed, int64_t n_orbits, int K, Norm nrm,
                                                    double step_frac, TrainSample* __restrict__ X,
                                                    int8_t* __restrict__ lab, unsigned long long* stats) {
    const double eps = nrm.t_eps;
    for (int64_t n = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; n < n_orbits;
         n += (int64_t)gridDim.x * blockDim.x) {
        uint64_t s = seed ^ (0xD1B54A32D192ED03ull * (uint64_t)(n + 1));
        const double lrc = log(double(nrm.rc_lo)) + unif(s) * (log(double(nrm.rc_hi)) - log(double(nrm.rc_lo)));
        const double rc = exp(lrc);
        // impact parameter: uniform in [0, b_max], or uniform in the transform t (dense near sqrt 27)
        double b;
        if (unif(s) < 0.5) {
            b = unif(s) * nrm.b_max;
        } else {
            const double t_lo = -log1p(1.0 / eps);
            const double t_hi = log1p((nrm.b_max / kSqrt27d - 1.0) / eps);
            const double tt = t_lo + unif(s) * (t_hi - t_lo);
            const double beta = (tt < 0 ? -1.0 : 1.0) * eps * expm1(fabs(tt));
            b = kSqrt27d * (1.0 + beta);
        }
        const double bgeo = rc / sqrt(1.0 - 2.0 / rc);  // a ray from rc reaches at most this b
        if (b > 0.999 * bgeo) b = unif(s) * 0.999 * bgeo;
        const double beta = b / kSqrt27d - 1.0;
        // initial state: static observer at rc, local angle alpha to the inward radial direction
        const double f = sqrt(1.0 - 2.0 / rc);
        const double sa = b * f / rc, ca = sqrt(1.0 - sa * sa);
        double vr = -ca * f, vt = sa;
        const double vn = rsqrt(vr * vr + vt * vt);
        vr *= vn;
        vt *= vn;
        const double h = rc * vt, m3h2 = -3.0 * h * h;
        const float x1 = float((lrc - log(double(nrm.rc_lo))) / (log(double(nrm.rc_hi)) - log(double(nrm.rc_lo))) * 2.0 - 1.0);
        const float x2 = float(bhr::orbit::b_transform<double>(beta, eps) * nrm.t_scale);
        // targets along the path (sigma ascending = path order); the last one is the exit
        double sig[kMaxK], uk[kMaxK];
        int nt = 0;
        bhr::orbit::Roots<double> R{};
        const double uc = 1.0 / rc;
        const bool turns = beta > 0.0;
        if (turns) {
            R = bhr::orbit::roots<double, 40>(beta);
            const double se = bhr::orbit::sigma_exit<double>(double(nrm.ue), R);
            for (int k = 0; k < K - 1; ++k) {  // uniform on [-1, exit], away from the turning point
                double sg;
                do {
                    sg = -1.0 + unif(s) * (1.0 + se);
                } while (fabs(sg) < 0.01);
                sig[nt++] = sg;
            }
            sig[nt++] = se;
            for (int a = 1; a < nt; ++a)  // insertion sort
                for (int c = a; c > 0 && sig[c] < sig[c - 1]; --c) {
                    const double tmp = sig[c];
                    sig[c] = sig[c - 1];
                    sig[c - 1] = tmp;
                }
            for (int k = 0; k < nt; ++k) uk[k] = bhr::orbit::u_of_sigma<double>(sig[k], uc, R);
        }
        // integrate
        P2 x{rc, 0.0}, v{vr, vt};
        double phi = 0.0, r = rc;
        int next = 0, status = 0;
        double phis[kMaxK];
        const double Ic = turns ? bhr::orbit::sweep_to_turn<double, 40>(uc, R) : 0.0;
        for (int it = 0; it < 400000; ++it) {
            const double vlen = sqrt(v.x * v.x + v.y * v.y);
            const double dt = step_frac * r / vlen, hdt = 0.5 * dt;
            const P2 k1v = acc2(x, m3h2), k1x = v;
            const P2 k2v = acc2({x.x + hdt * k1x.x, x.y + hdt * k1x.y}, m3h2), k2x{v.x + hdt * k1v.x, v.y + hdt * k1v.y};
            const P2 k3v = acc2({x.x + hdt * k2x.x, x.y + hdt * k2x.y}, m3h2), k3x{v.x + hdt * k2v.x, v.y + hdt * k2v.y};
            const P2 k4v = acc2({x.x + dt * k3x.x, x.y + dt * k3x.y}, m3h2), k4x{v.x + dt * k3v.x, v.y + dt * k3v.y};
            const double s6 = dt / 6.0;
            const P2 xn{x.x + s6 * (k1x.x + 2 * k2x.x + 2 * k3x.x + k4x.x), x.y + s6 * (k1x.y + 2 * k2x.y + 2 * k3x.y + k4x.y)};
            const P2 vnw{v.x + s6 * (k1v.x + 2 * k2v.x + 2 * k3v.x + k4v.x), v.y + s6 * (k1v.y + 2 * k2v.y + 2 * k3v.y + k4v.y)};
            const double rn = sqrt(xn.x * xn.x + xn.y * xn.y);
            const double dphi = atan2(x.x * xn.y - x.y * xn.x, x.x * xn.x + x.y * xn.y);
            const bool in0 = (x.x * v.x + x.y * v.y) < 0.0;
            const bool in1 = (xn.x * vnw.x + xn.y * vnw.y) < 0.0;
            // targets reached in this step: ingoing leg (sigma < 0): r falls through 1/u while ingoing;
            // outgoing leg: r rises through 1/u while outgoing
            while (turns && next < nt) {
                const double Rk = 1.0 / uk[next];
                bool hit;
                if (sig[next] < 0.0) hit = in0 && rn <= Rk && r > Rk;
                else hit = !in1 && rn >= Rk && r < Rk;
                if (!hit) break;
                phis[next] = phi + hermite_angle(x, {v.x * dt, v.y * dt}, xn, {vnw.x * dt, vnw.y * dt}, r, rn, Rk);
                ++next;
            }
            (void)in1;
            x = xn;
            v = vnw;
            r = rn;
            phi += dphi;
            if (r < 2.0001) {
                status = 2;
                break;
            }
            if (r > 1.0 / double(nrm.ue) && !(x.x * v.x + x.y * v.y < 0.0)) {
                status = 1;
                break;
            }
        }
        const int64_t base = n * K;
        // orbits well inside the fallback band are never queried: keep them out of the regression
        const bool in_band = fabs(beta) < 0.5 * double(nrm.band) / kSqrt27d;
        if (status == 1 && turns && next == nt && !in_band) {
            for (int k = 0; k < nt; ++k) {
                const double bl = bhr::orbit::base_blend<double>(beta);
                const double I = bhr::orbit::base_sweep<double>(uk[k], R, bl);
                const double Icb = bhr::orbit::base_sweep<double>(uc, R, bl);
                const double base_phi = sig[k] < 0.0 ? Icb - I : Icb + I;
                X[base + k] = TrainSample{x1, x2, float(sig[k]), float((phis[k] - base_phi) / nrm.y_scale)};
                lab[base + k] = 0;
            }
            atomicAdd(&stats[0], 1ull);
        } else if (status == 2) {
            for (int k = 0; k < K; ++k) {
                X[base + k] = TrainSample{x1, x2, 1.0f, 0.0f};
                lab[base + k] = 1;
            }
            atomicAdd(&stats[1], 1ull);
        } else {
            for (int k = 0; k < K; ++k) {
                X[base + k] = TrainSample{x1, x2, 1.0f, 0.0f};
                lab[base + k] = 2;
            }
            atomicAdd(&stats[2], 1ull);
        }
        (void)Ic;
    }
}

// ---------------------------------------------------------------------------------------
// training: fused forward + backward per warp (32 samples). Each warp adds its tile's gradients
// with global reductions into one of kGradCopies copies of the gradient buffer (fire-and-forget
// at L2, spread over the copies' addresses); k_adam sums the copies and zeroes them. Summing in
// shared memory first made every warp wait on its 8,706 shared-memory additions (61.5 against
// 38.5 us per step at batch 16,384; one copy in global memory: 66.8 us, from contention)

constexpr int kTrainWarps = 4;

struct WarpAct {                      // per warp, BF16 [32 rows][kLd]
    __nv_bfloat16 z1[32 * kLd], h1[32 * kLd], z2[32 * kLd], h2[32 * kLd], dz2[32 * kLd], dz3[32 * kLd];
    float4 x[32];
    float y[32];
    int lab[32];
};

struct TrainSmem {
    SmemNet N;
    SmemNetT T;
    float loss[3];                    // sum of squared y error, sum of BCE, y-sample count
    WarpAct w[kTrainWarps];
};

// sum over the 8 groups g (lanes with equal t) of a value, result valid in lanes with g == 0
__device__ __forceinline__ float sum_over_g(float v) {
    v += __shfl_xor_sync(0xffffffffu, v, 4);
    v += __shfl_xor_sync(0xffffffffu, v, 8);
    v += __shfl_xor_sync(0xffffffffu, v, 16);
    return v;
}

// dW[out][in] += sum over the warp's 32 rows of dz[row][out] * h[row][in] (BF16 MMA, K = 32 rows)
__device__ void mma_weight_grad(const __nv_bfloat16* dz, const __nv_bfloat16* h, float* gW, int g, int t) {
#pragma unroll 1
    for (int mo = 0; mo < 4; ++mo) {
        float C[8][4];
#pragma unroll
        for (int j = 0; j < 8; ++j) C[j][0] = C[j][1] = C[j][2] = C[j][3] = 0.f;
#pragma unroll
        for (int ki = 0; ki < 2; ++ki) {
            const int r0 = 16 * ki + 2 * t;
            const int o0 = 16 * mo + g;
            uint32_t A[4];
            A[0] = pack2(dz[r0 * kLd + o0], dz[(r0 + 1) * kLd + o0]);
            A[1] = pack2(dz[r0 * kLd + o0 + 8], dz[(r0 + 1) * kLd + o0 + 8]);
            A[2] = pack2(dz[(r0 + 8) * kLd + o0], dz[(r0 + 9) * kLd + o0]);
            A[3] = pack2(dz[(r0 + 8) * kLd + o0 + 8], dz[(r0 + 9) * kLd + o0 + 8]);
            const uint32_t (&Ar)[4] = A;
#pragma unroll
            for (int j = 0; j < 8; ++j) {
                const int n0 = 8 * j + g;
                const uint32_t b0 = pack2(h[r0 * kLd + n0], h[(r0 + 1) * kLd + n0]);
                const uint32_t b1 = pack2(h[(r0 + 8) * kLd + n0], h[(r0 + 9) * kLd + n0]);
                mma_bf16(C[j], Ar, b0, b1);
            }
        }
#pragma unroll
        for (int j = 0; j < 8; ++j) {
            const int o = 16 * mo + g, i = 8 * j + 2 * t;
            atomicAdd(&gW[o * kH + i], C[j][0]);
            atomicAdd(&gW[o * kH + i + 1], C[j][1]);
            atomicAdd(&gW[(o + 8) * kH + i], C[j][2]);
            atomicAdd(&gW[(o + 8) * kH + i + 1], C[j][3]);
        }
    }
}

__global__ void __launch_bounds__(32 * kTrainWarps, 1) k_train_step(
    const float* __restrict__ P, const TrainSample* __restrict__ X, const int8_t* __restrict__ lab,
    int64_t n_samples, const int64_t* __restrict__ idx, int batch, uint64_t seed, float w_u, float w_c,
    float* __restrict__ G, float* __restrict__ loss_out) {
    extern __shared__ __align__(16) unsigned char smem_raw[];
    TrainSmem& S = *reinterpret_cast<TrainSmem*>(smem_raw);
    load_net(S.N, &S.T, P);
    if (threadIdx.x < 3) S.loss[threadIdx.x] = 0.f;
    __syncthreads();
    const SmemNet& N = S.N;
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31, g = lane >> 2, t = lane & 3;
    WarpAct& W = S.w[warp];
    float* const Gw = G + size_t((blockIdx.x * kTrainWarps + warp) % kGradCopies) * kNParams;
    const float inv_b = 1.0f / float(batch);
    float l_y = 0.f, l_c = 0.f, n_y = 0.f;
    const int tiles = batch / 32;
    for (int tile = blockIdx.x * kTrainWarps + warp; tile < tiles; tile += gridDim.x * kTrainWarps) {
        // ---- load 32 samples
        const int64_t e = (int64_t)tile * 32 + lane;
        int64_t si;
        if (idx) si = idx[e];
        else si = int64_t(splitmix(seed ^ (0x9E3779B97F4A7C15ull * uint64_t(e + 1))) % uint64_t(n_samples));
        const TrainSample ts = X[si];
        W.x[lane] = make_float4(ts.x1, ts.x2, ts.sigma, 0.f);
        W.y[lane] = ts.y;
        W.lab[lane] = lab[si];
        __syncwarp();
#pragma unroll 1
        for (int mt = 0; mt < 2; ++mt) {
            const int ra = 16 * mt + g, rb = ra + 8;
            uint32_t A[4][4];
            float C[8][4];
            // ---- forward
            layer1<true>(N, W.x[ra], W.x[rb], A, t, W.z1, W.h1, ra, rb);
            mma_layer(N.w2, N.b2, A, C, g, t);
#pragma unroll
            for (int j = 0; j < 8; ++j) {
                const int f = 8 * j + 2 * t;
                W.z2[ra * kLd + f] = __float2bfloat16_rn(C[j][0]);
                W.z2[ra * kLd + f + 1] = __float2bfloat16_rn(C[j][1]);
                W.z2[rb * kLd + f] = __float2bfloat16_rn(C[j][2]);
                W.z2[rb * kLd + f + 1] = __float2bfloat16_rn(C[j][3]);
            }
            act_pack(C, A);
#pragma unroll
            for (int i = 0; i < 4; ++i) {
                const int f = 16 * i + 2 * t;
                st_pair(&W.h2[ra * kLd + f], A[i][0]);
                st_pair(&W.h2[rb * kLd + f], A[i][1]);
                st_pair(&W.h2[ra * kLd + f + 8], A[i][2]);
                st_pair(&W.h2[rb * kLd + f + 8], A[i][3]);
            }
            float Z3[8][4];
            mma_layer(N.w3, N.b3, A, Z3, g, t);
            float o[2][2];
            out_layer(N, Z3, o, t);
            // ---- loss and output gradients (rows ra, rb)
            float dy[2], dc[2];
#pragma unroll
            for (int rr = 0; rr < 2; ++rr) {
                const int row = rr ? rb : ra;
                const int lb = W.lab[row];
                const bool yok = lb == 0;
                const float err = o[rr][0] - W.y[row];
                dy[rr] = yok ? 2.0f * w_u * err * inv_b : 0.f;
                const float target = lb == 1 ? 1.f : 0.f;
                const float p = 1.0f / (1.0f + __expf(-o[rr][1]));
                const bool cok = lb != 2;
                dc[rr] = cok ? w_c * (p - target) * inv_b : 0.f;
                if (t == 0) {
                    if (yok) {
                        l_y += err * err;
                        n_y += 1.f;
                    }
                    if (cok) l_c += fmaxf(o[rr][1], 0.f) - o[rr][1] * target + log1pf(__expf(-fabsf(o[rr][1])));
                }
            }
            // ---- output layer gradients and dz3
            float D[8][4];
#pragma unroll
            for (int j = 0; j < 8; ++j) {
                const int f = 8 * j + 2 * t;
                float gw[2][2] = {{0.f, 0.f}, {0.f, 0.f}}, gb[2] = {0.f, 0.f};
                const uint32_t sa = silu_pair_h(0.5f * Z3[j][0], 0.5f * Z3[j][1]);
                const uint32_t sb = silu_pair_h(0.5f * Z3[j][2], 0.5f * Z3[j][3]);
                const float hv[4] = {bf_lo(sa), bf_hi(sa), bf_lo(sb), bf_hi(sb)};
#pragma unroll
                for (int c = 0; c < 4; ++c) {
                    const int rr = c >> 1, ff = f + (c & 1);
                    const float h3 = hv[c];
                    gw[0][c & 1] += dy[rr] * h3;
                    gw[1][c & 1] += dc[rr] * h3;
                    const float dh = dy[rr] * N.w4[ff] + dc[rr] * N.w4[kH + ff];
                    D[j][c] = dh * silu_grad(Z3[j][c]);
                    gb[c & 1] += D[j][c];
                }
                float v00 = sum_over_g(gw[0][0]), v01 = sum_over_g(gw[0][1]);
                float v10 = sum_over_g(gw[1][0]), v11 = sum_over_g(gw[1][1]);
                float b0 = sum_over_g(gb[0]), b1 = sum_over_g(gb[1]);
                if (g == 0) {
                    atomicAdd(&Gw[kW4 + f], v00);
                    atomicAdd(&Gw[kW4 + f + 1], v01);
                    atomicAdd(&Gw[kW4 + kH + f], v10);
                    atomicAdd(&Gw[kW4 + kH + f + 1], v11);
                    atomicAdd(&Gw[kB3 + f], b0);
                    atomicAdd(&Gw[kB3 + f + 1], b1);
                }
                W.dz3[ra * kLd + f] = __float2bfloat16_rn(D[j][0]);
                W.dz3[ra * kLd + f + 1] = __float2bfloat16_rn(D[j][1]);
                W.dz3[rb * kLd + f] = __float2bfloat16_rn(D[j][2]);
                W.dz3[rb * kLd + f + 1] = __float2bfloat16_rn(D[j][3]);
            }
            {
                float gb0 = dy[0] + dy[1], gb1 = dc[0] + dc[1];
                gb0 = sum_over_g(gb0);
                gb1 = sum_over_g(gb1);
                if (lane == 0) {
                    atomicAdd(&Gw[kB4], gb0);
                    atomicAdd(&Gw[kB4 + 1], gb1);
                }
            }
            // ---- dh2 = dz3 W3, dz2 = dh2 silu'(z2)
            pack_only(D, A);
            mma_layer(S.T.w3t, nullptr, A, C, g, t);
#pragma unroll
            for (int j = 0; j < 8; ++j) {
                const int f = 8 * j + 2 * t;
                float gb[2] = {0.f, 0.f};
#pragma unroll
                for (int c = 0; c < 4; ++c) {
                    const int row = (c >> 1) ? rb : ra, ff = f + (c & 1);
                    C[j][c] *= silu_grad(__bfloat162float(W.z2[row * kLd + ff]));
                    gb[c & 1] += C[j][c];
                    W.dz2[row * kLd + ff] = __float2bfloat16_rn(C[j][c]);
                }
                const float b0 = sum_over_g(gb[0]), b1 = sum_over_g(gb[1]);
                if (g == 0) {
                    atomicAdd(&Gw[kB2 + f], b0);
                    atomicAdd(&Gw[kB2 + f + 1], b1);
                }
            }
            // ---- dh1 = dz2 W2, dz1 = dh1 silu'(z1); layer-1 gradients in FP32
            pack_only(C, A);
            float E[8][4];
            mma_layer(S.T.w2t, nullptr, A, E, g, t);
            const float4 xa = W.x[ra], xb = W.x[rb];
#pragma unroll
            for (int j = 0; j < 8; ++j) {
#pragma unroll
                for (int h = 0; h < 2; ++h) {
                    const int f = 8 * j + 2 * t + h;
                    const float da = E[j][h] * silu_grad(__bfloat162float(W.z1[ra * kLd + f]));
                    const float db = E[j][2 + h] * silu_grad(__bfloat162float(W.z1[rb * kLd + f]));
                    const float g0 = sum_over_g(da * xa.x + db * xb.x);
                    const float g1 = sum_over_g(da * xa.y + db * xb.y);
                    const float g2 = sum_over_g(da * xa.z + db * xb.z);
                    const float gb = sum_over_g(da + db);
                    if (g == 0) {
                        atomicAdd(&Gw[kW1 + 3 * f], g0);
                        atomicAdd(&Gw[kW1 + 3 * f + 1], g1);
                        atomicAdd(&Gw[kW1 + 3 * f + 2], g2);
                        atomicAdd(&Gw[kB1 + f], gb);
                    }
                }
            }
        }
        __syncwarp();
        // ---- hidden weight gradients over the 32 rows
        mma_weight_grad(W.dz3, W.h2, &Gw[kW3], g, t);
        mma_weight_grad(W.dz2, W.h1, &Gw[kW2], g, t);
        __syncwarp();
    }
    if (t == 0) {
        atomicAdd(&S.loss[0], l_y);
        atomicAdd(&S.loss[1], l_c);
        atomicAdd(&S.loss[2], n_y);
    }
    __syncthreads();
    if (threadIdx.x < 3) atomicAdd(&loss_out[threadIdx.x], S.loss[threadIdx.x]);
}

__global__ void k_adam(float* __restrict__ p, float* __restrict__ gr, float* __restrict__ m,
                       float* __restrict__ v, int step, float lr, float b1, float b2, float eps) {
    const int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= kNParams) return;
    float g = 0.f;
    for (int r = 0; r < kGradCopies; ++r) {
        g += gr[size_t(r) * kNParams + k];
        gr[size_t(r) * kNParams + k] = 0.f;  // zero for the next step
    }
    const float mk = b1 * m[k] + (1.f - b1) * g;
    const float vk = b2 * v[k] + (1.f - b2) * g * g;
    m[k] = mk;
    v[k] = vk;
    const float mh = mk / (1.f - powf(b1, float(step)));
    const float vh = vk / (1.f - powf(b2, float(step)));
    p[k] -= lr * mh / (sqrtf(vh) + eps);
}

// Plain forward pass over n queries (tests and the gradient check) on the tcgen05 network: one
// warpgroup per block, 128 queries per tile. *status is set to 1 if a tensor-core wait ran out
// (the tile's outputs are then NaN and the block stops). ctl.withhold is the self-test of that
// path: no MMA is issued, so every wait runs out with nothing in flight.
__global__ void __launch_bounds__(128, 4) k_mlp_infer(const float* __restrict__ P, const float4* __restrict__ q,
                                                      float2* __restrict__ out, int n, int* __restrict__ status,
                                                      const tc::TileCtl ctl) {
    extern __shared__ __align__(16) unsigned char smem_raw[];
    tc::Net& N = *reinterpret_cast<tc::Net*>(smem_raw);
    tc::L1& l1 = *reinterpret_cast<tc::L1*>(smem_raw + sizeof(tc::Net));
    tc::Tile& T = *reinterpret_cast<tc::Tile*>(smem_raw + sizeof(tc::Net) + sizeof(tc::L1));
    __shared__ uint32_t tmem_slot;
    __shared__ int fail;
    tc::load_net(N, P, false, 0.f);
    tc::load_l1(l1, P);
    if (threadIdx.x == 0) {
        tc::mbar_init(tc::smem_u32(&T.mbar), 1);
        fail = 0;
    }
    if (threadIdx.x < 32) tc::tmem_alloc(tc::smem_u32(&tmem_slot), tc::kTmemCols);
    tc::fence_smem_async();
    tc::fence_before();
    __syncthreads();
    tc::fence_after();
    const uint32_t tmem = tmem_slot;
    uint32_t phase = 0;
    for (int t0 = blockIdx.x * tc::kRows; t0 < n; t0 += gridDim.x * tc::kRows) {
        const int row = t0 + int(threadIdx.x);
        const float4 x = row < n ? q[row] : make_float4(0.f, 0.f, 0.f, 0.f);
        float2 o;
        const bool ok = tc::mlp_tile_l1f(N, l1, T, tmem, int(threadIdx.x), 1, phase, x, o, ctl);
        if (!ok) fail = 1;
        if (row < n) out[row] = ok ? o : make_float2(__int_as_float(0x7fc00000), __int_as_float(0x7fc00000));
        __syncthreads();
        if (fail) break;
    }
    if (fail && threadIdx.x == 0) atomicExch(status, 1);
    tc::fence_before();
    __syncthreads();
    if (threadIdx.x < 32) {
        tc::fence_after();
        tc::tmem_dealloc(tmem, tc::kTmemCols);
    }
}

// ---------------------------------------------------------------------------------------
// inference: one warp traces 32 rays at a time, in phases that hand state on through shared
// memory, so that no lane waits on another lane's crossing loop. Within a view, everything an
// escaping orbit's record needs except its orientation is a function of the impact parameter
// alone (the camera radius and the rule are the view's): the exit angle with the network's
// residual, the escape direction in the orbital plane after farFieldDirection at the exit, the
// angle to the turning point, the periapsis and the capture logit. The view's exit table
// (built by k_tables before the pass) holds them per point of x2, and its crossing table the
// network's residual for crossing queries. The rays interpolate them:
//   1  per ray (lane): setup and routing, the orbital plane, the exit table, and the disk-plane
//      crossings inside the disk's angle range (candidates, found without inverting the orbit);
//      captured orbits take the exact one-real-root form
//   2  per candidate, spread over the warp's lanes: roots, inversion of the closed form u(phi),
//      the crossing table's residual, the crossing radius and azimuth
//   3  per ray: the escape direction in 3-D and the record
// The surrogate variant without the network (kNet false) builds the same tables from the
// converged closed form (orbit::Baseline<false>) and reads no crossing table.

constexpr int kInferWarps = 8;
constexpr int kMaxCand = 3;                   // crossings kept per ray (the record holds 3)
constexpr int kCapDup = 3;                    // R_F duplication steps of the captured-orbit closed form
constexpr uint32_t kCapBit = 1u << 26;        // stage info: the ray's orbit is captured

struct RayStage {  // per warp, structure of arrays over its 32 rays
    float s0[32], s1[32], s2[32], s3[32];  // captured orbit: u1, A, k^2, K
    float ic[32];      // angle camera -> turning point (escaping), F(camera) (captured)
    float phin[32], x2[32], beta[32];
    float nx[32], nz[32];  // the nodal line's direction in the disk plane (x, z; unnormalised): crossing k lies
                           // at its end (-1)^k
    float b[32];
    uint32_t info[32];  // bits 0-1 candidates, 2 surrogate, 3-10 plane crossings, 11+5c candidate c (k | leg << 4),
                        // 26 captured orbit
};

struct InferSmem {
    RayStage st[kInferWarps];
    int task[kInferWarps][32 * kMaxCand];     // owner lane << 2 | candidate
    float tu[kInferWarps][32 * kMaxCand];     // the crossing radius (< 0: outside the disk)
    float tphi[kInferWarps][32 * kMaxCand];   // azimuth of the crossing
};

__device__ __forceinline__ unsigned long long warp_append_ull(unsigned long long* ctr) {
    const unsigned m = __activemask();
    const int leader = __ffs(m) - 1;
    const int lane = threadIdx.x & 31;
    unsigned long long base = 0;
    if (lane == leader) base = atomicAdd(ctr, (unsigned long long)__popc(m));
    base = __shfl_sync(m, base, leader);
    return base + __popc(m & ((1u << lane) - 1u));
}

// sin and cos of x (|x| < 1e4): Cody-Waite reduction by pi/2 with a two-part constant, then
// Taylor polynomials on [-pi/4, pi/4] (truncation below 3e-9) and the quadrant rotation.
__device__ __forceinline__ void sincos_rr(float x, float* sn, float* cs) {
    const float k = rintf(x * 0.63661977236758134f);
    float r = fmaf(-k, 1.57079637050628662f, x);
    r = fmaf(k, 4.37113900018624e-8f, r);
    const float r2 = r * r;
    const float sp = r * fmaf(r2, fmaf(r2, fmaf(r2, fmaf(r2, 2.7557319e-6f, -1.9841270e-4f), 8.3333333e-3f),
                                       -1.6666667e-1f), 1.0f);
    const float cp = fmaf(r2, fmaf(r2, fmaf(r2, fmaf(r2, 2.4801587e-5f, -1.3888889e-3f), 4.1666667e-2f), -0.5f), 1.0f);
    const int q = int(k) & 3;
    const float s0 = (q & 1) ? cp : sp, c0 = (q & 1) ? sp : cp;
    *sn = (q & 2) ? -s0 : s0;
    *cs = ((q + 1) & 2) ? -c0 : c0;
}

// Impact parameter of pixel (i, j) in FP64, for rays near the photon sphere, where the FP32
// value (relative error ~1e-7) would move the exit angle by more than the error budget:
// b = r_cam sin(alpha) / sqrt(1 - 2 / r_cam) (Geodesic.h:50-54), alpha the angle between the
// ray and the radial direction, from the unnormalised pixel direction (blackhole.frag:68-72)
// in double. The view constants arrive in double. Out of line: rare, and its FP64 code would
// otherwise crowd the instruction cache.
__device__ __noinline__ double impact_parameter_fp64(const DevView& w, const Fp64Cam& fc, int i, int j) {
    const double pxx = double(i) + 0.5 + double(w.jitter[0]);
    const double pxy = double(j) + 0.5 + double(w.jitter[1]);
    const double th = double(w.tan_half);
    const double cx = (pxx * fc.inv_w2 - 1.0) * th * fc.aspect_d;
    const double cy = (pxy * fc.inv_h2 - 1.0) * th;
    const double dx = double(w.basis[0]) * cx + double(w.basis[3]) * cy - double(w.basis[6]);
    const double dy = double(w.basis[1]) * cx + double(w.basis[4]) * cy - double(w.basis[7]);
    const double dz = double(w.basis[2]) * cx + double(w.basis[5]) * cy - double(w.basis[8]);
    const double* rh = fc.rhat_d;
    const double px = rh[1] * dz - rh[2] * dy, py = rh[2] * dx - rh[0] * dz, pz = rh[0] * dy - rh[1] * dx;
    const double s2 = (px * px + py * py + pz * pz) / (dx * dx + dy * dy + dz * dz);
    return fc.b_scale_d * ::sqrt(s2);
}

// The band rays of every view, before the surrogate pass (one warp per searched pixel row).
// Along row j the pixel direction is d(cx) = cx R + (cy U - B) (the camera basis' columns), and
// cos^2 of its angle from the hole, (rhat . d)^2 / |d|^2, is at least c exactly where the
// quadratic (rhat . d)^2 - c |d|^2 is non-negative: between its two roots, since the hole lies
// well inside the field of view (bhr::surr::band_rows). The band's pixels lie between the
// roots for c_out (the larger angle) and outside those for c_in; two pixels of margin on each
// end, and a b range twice the band's, leave every band ray inside the searched pixels, which
// the warp's lanes take 32 at a time. Everything runs in FP32 (FP64 runs at a small fraction
// of the FP32 rate here): the roots, and the band test on the FP32 impact parameter, which is
// within 2e-6 of the FP64 one in beta near the photon sphere. Only rays within kBandEdge of the
// band's edge take the pass's own FP64 test. A band ray joins its view's list and sets its bit
// in the view's mask (the pass skips those rays). A ray the search missed would still be found
// by the pass and go to the fallback list: the mask, not the test, decides who answers a ray.
constexpr float kBandEdge = 1e-5f;
__global__ void __launch_bounds__(128) k_band_list(const __grid_constant__ BandBatch bb) {
    const int t = blockIdx.x * 4 + (threadIdx.x >> 5), lane = threadIdx.x & 31;
    if (t >= bb.total_rows) return;
    int vi = 0;
    while (vi + 1 < bb.nviews && t >= bb.v[vi + 1].row0) ++vi;
    const BandView& bv = bb.v[vi];
    const int j = t - bv.row0;
    if (j >= bv.rows) return;
    const DevView& w = bv.view;
    const BandRows& Q = bv.q;
    // the row's quadratic in cx: (a cx + a0)^2 - c (RR cx^2 + 2 rd cx + dd)
    const float th = w.tan_half;
    const float cy = ((float(j) + 0.5f + w.jitter[1]) * (2.0f / float(w.height)) - 1.0f) * th;
    const float a = Q.a, a0 = cy * Q.rhU - Q.rhB;
    const float rd = cy * Q.RU - Q.RB, dd = cy * cy * Q.UU - 2.0f * cy * Q.UB + Q.BB;
    const float sx = th * w.aspect;  // cx = ((i + 0.5 + jitter) 2 / W - 1) sx
    auto roots = [&](float c, float* lo, float* hi) {
        const float A2 = a * a - c * Q.RR, A1 = 2.0f * (a * a0 - c * rd), A0 = a0 * a0 - c * dd;
        float disc = A1 * A1 - 4.0f * A2 * A0;
        if (disc < 0.0f && disc > -1e-5f) disc = 0.0f;  // a tangent row: the margin covers the rounding
        if (!(A2 < 0.0f) || !(disc >= 0.0f)) return false;
        const float q = sqrtf(disc);
        const float x1 = (-A1 + q) / (2.0f * A2), x2 = (-A1 - q) / (2.0f * A2);
        auto col = [&](float cx) { return (cx / sx + 1.0f) * (0.5f * float(w.width)) - 0.5f - w.jitter[0]; };
        *lo = col(fminf(x1, x2));
        *hi = col(fmaxf(x1, x2));
        return true;
    };
    float p1, p2, q1 = 0.0f, q2 = -1.0f;
    if (!roots(Q.c_out, &p1, &p2)) return;
    const bool inner = roots(Q.c_in, &q1, &q2);
    constexpr float kMargin = 2.0f;
    auto clampc = [&](float x) { return int(fminf(fmaxf(x, -1.0f), float(w.width))); };
    int seg[2][2] = {{0, -1}, {0, -1}};
    if (inner && q2 - q1 > 2.0f * kMargin) {
        seg[0][0] = clampc(floorf(p1 - kMargin));
        seg[0][1] = clampc(ceilf(q1 + kMargin));
        seg[1][0] = clampc(floorf(q2 - kMargin));
        seg[1][1] = clampc(ceilf(p2 + kMargin));
    } else {
        seg[0][0] = clampc(floorf(p1 - kMargin));
        seg[0][1] = clampc(ceilf(p2 + kMargin));
    }
    const float beta_band = bb.band / kSqrt27f;
    unsigned long long* cnt = &bb.qb[2 * vi].fb_count;
    for (int sgi = 0; sgi < 2; ++sgi) {
        const int i0 = max(seg[sgi][0], 0), i1 = min(seg[sgi][1], w.width - 1);
        for (int i = i0 + lane; i <= i1; i += 32) {
            const RayInit<float> ri = setup_ray<float>(w, bb.rule, i, j);
            const float ab = fabsf(ri.b * (1.0f / kSqrt27f) - 1.0f);
            bool in = ab < beta_band - kBandEdge;
            if (!in && ab < beta_band + kBandEdge) {  // at the edge: the pass's FP64 test
                const double bd = impact_parameter_fp64(w, bv.fc, i, j);
                in = fabsf(float(bd * (1.0 / kSqrt27d) - 1.0)) < beta_band;
            }
            if (!in) continue;
            const int ray = j * w.width + i;
            const unsigned long long k = atomicAdd(cnt, 1ull);
            if (k < (unsigned long long)kBandCap) {
                bv.list[k] = ray;
                atomicOr(bv.mask + (ray >> 5), 1u << (ray & 31));
            } else {
                atomicAdd(cnt, ~0ull);  // minus one: the count settles at kBandCap; this ray takes the fallback list
            }
        }
    }
}

// Phase-1 work of a captured orbit, out of line: it runs for the rays of the shadow only, and
// inlined it would crowd the instruction cache of every warp.
struct CapStage {
    float u1, A, k2, K;  // the orbit (orbit::CapOrbit without c)
    float Ic;            // F(theta(u_camera))
    float phi0;          // angle from the camera to the capture radius
    float Ilo, Ihi;      // angles from the camera to 1.03 r_out and 0.97 r_in (empty range: Ilo > Ihi)
};

__device__ __noinline__ CapStage cap_stage(float beta, float uc, float capture_r, float disk_inner, float disk_outer,
                                           bool range) {
    const orbit::CapOrbit<float> C = orbit::cap_orbit<float, kCapDup>(beta);
    CapStage o;
    o.u1 = C.u1;
    o.A = C.A;
    o.k2 = C.k2;
    o.K = C.K;
    const float s2a = rsqrtf(2.0f * C.A);
    o.Ic = orbit::cap_F<float, kCapDup>(uc, C);
    o.phi0 = (orbit::cap_F<float, kCapDup>(1.0f / capture_r, C) - o.Ic) * s2a;
    o.Ilo = 1.f;
    o.Ihi = 0.f;
    if (range) {
        // crossing k lies in [0.97 r_in, 1.03 r_out] iff phi_k lies between the angles from the
        // camera to those radii on the way in (clipped to the camera and the capture radius)
        const float ua = fmaxf(1.0f / (disk_outer * 1.03f), uc);
        const float ub = fminf(1.0f / (disk_inner * 0.97f), 1.0f / capture_r);
        if (ua < ub) {
            o.Ilo = (orbit::cap_F<float, kCapDup>(ua, C) - o.Ic) * s2a;
            o.Ihi = (orbit::cap_F<float, kCapDup>(ub, C) - o.Ic) * s2a;
        }
    }
    return o;
}

// u of a captured orbit at angle phk from the camera: Newton on phi(u) = phk with
// dphi/du = 1 / sqrt(P(u)), kept in [u_camera, 1 / capture_r]. Out of line for the same reason.
__device__ __noinline__ float cap_invert(float u1, float A, float k2, float K, float b, float Fc, float phk, float uc,
                                         float capture_r, float disk_inner, float disk_outer) {
    orbit::CapOrbit<float> C;
    C.u1 = u1;
    C.A = A;
    C.k2 = k2;
    C.K = K;
    const float cb = 1.0f / b;
    C.c = cb * cb;
    const float s2a = rsqrtf(2.0f * A);
    const float uh = 1.0f / capture_r;
    float u = fminf(fmaxf(0.5f * (1.0f / (disk_inner * 0.97f) + 1.0f / (disk_outer * 1.03f)), uc), uh);
#pragma unroll 1
    for (int it = 0; it < 6; ++it) {
        const float f = (orbit::cap_F<float, kCapDup>(u, C) - Fc) * s2a - phk;
        const float P = fmaxf(2.0f * u * u * u - u * u + C.c, 0.f);
        u = fminf(fmaxf(u - f * sqrtf(P), uc), uh);
    }
    return u;
}

// Writes point i's value f into the four cubic entries (f_j .. f_{j+3}) that hold it.
__device__ __forceinline__ void put_cubic(float* T, int i, float f) {
#pragma unroll
    for (int d = 0; d < 4; ++d) {
        const int j = i - d;
        if (j >= 0 && j <= kExitTableN - 4) T[4 * j + d] = f;
    }
}

// Writes point i's values (a, c) into the pair entries i (slots 0, 2 or, with kAdj, 0, 1) and
// i - 1 (slots 1, 3 or 2, 3): entry m holds points m and m + 1; the last entry repeats its point.
template <bool kAdj>
__device__ __forceinline__ void put_pair(float* T, int i, float a, float c) {
    constexpr int s0 = 0, s1 = kAdj ? 1 : 2, t0 = kAdj ? 2 : 1, t1 = 3;
    T[4 * i + s0] = a;
    T[4 * i + s1] = c;
    if (i > 0) {
        T[4 * (i - 1) + t0] = a;
        T[4 * (i - 1) + t1] = c;
    }
    if (i == kExitTableN - 1) {
        T[4 * i + t0] = a;
        T[4 * i + t1] = c;
    }
}

// The in-plane escape direction (its angle from e1, e1 = the camera direction and e2 the ray's
// tangential direction) of an escaping orbit that leaves the march at u = ue at angle phi0 from
// the camera: the exit position and velocity (energy integral of x'' = -3 h^2 x / r^5 with
// h^2 = b^2 / (1 + 2 b^2 / r_cam^3)), then farFieldDirection (geodesic.glsl:43-53) there,
// measured from the radial direction at the exit, so that the angle stays continuous in b.
__device__ __forceinline__ float escape_angle(float phi0, float ue, const orbit::Roots<float>& Rt, float b,
                                              float two_over_r3) {
    float sp, cp;
    sincos_rr(phi0, &sp, &cp);
    const float re = 1.0f / ue;
    const V3<float> xe{re * cp, re * sp, 0.f};
    const float sP = orbit::dudphi<float>(ue, Rt);
    V3<float> Tv{sP * re * re * cp - re * sp, sP * re * re * sp + re * cp, 0.f};
    const float b2 = b * b;
    const float h2 = b2 / (1.0f + b2 * two_over_r3);
    const float vmag = sqrtf(fmaxf(1.0f - h2 * two_over_r3 + 2.0f * h2 * ue * ue * ue, 1e-12f));
    const float Ti = vmag * rsqrtf(dot3(Tv, Tv));
    Tv = {Tv.x * Ti, Tv.y * Ti, 0.f};
    const V3<float> d = far_field_dir(xe, Tv, h2);
    return phi0 + atan2f(cp * d.y - sp * d.x, cp * d.x + sp * d.y);
}

// The exit table (layout in surrogate.cuh) of the non-learned variant: per point of the escaping
// half, the beta it encodes (the inverse of the x2 transform) and from it the roots, the exit u of
// the rule (with kTol, of each branch of the tolerance escape), the converged closed form from the
// camera to the turning point, to the exit and to the disk's radii, the exit angle and the escape
// direction (escape_angle). Each point is written into every entry it belongs to. (The learned
// variant's tables, with the network, come from k_tables.)
template <bool kTol>
__global__ void __launch_bounds__(256) k_exit_table_cf(const __grid_constant__ SurrView sv, float4* __restrict__ table) {
    constexpr int kQ = kTol ? 2 : 1;  // exits per point: one per branch of the rule's exit
    const Norm& nm = sv.norm;
    float* T = reinterpret_cast<float*>(table);
    constexpr float kPi = 3.14159265358979f;
    using B = orbit::Baseline<false>;
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < kExitTableN; i += gridDim.x * blockDim.x) {
        const float x2 = fmaf(float(i), sv.tab_h[1], sv.tab_lo[1]);
        const float beta = fmaxf(nm.t_eps * expm1f(x2 / nm.t_scale), 1e-7f);
        const float b = kSqrt27f * (1.0f + beta);
        const orbit::Roots<float> Rt = orbit::roots<float, 4>(beta);
        float ue[2];
        if (kTol) {
            ue[0] = fminf(sv.u_esc_min, Rt.u2);
            ue[1] = orbit::exit_u_tol<float>(b, sv.rule.esc_tol, 1.0f, Rt.u2);
        } else {
            ue[0] = nm.ue;
        }
        const float Ic = B::template sweep<float>(sv.uc, Rt, beta);
        for (int r = 0; r < kQ; ++r) {
            const float phi0 = Ic + B::template sweep<float>(ue[r], Rt, beta);
            const float psi = escape_angle(phi0, ue[r], Rt, b, sv.view.two_over_r3);
            put_cubic(T + 4 * (r ? kExitPsiB : kExitPsi), i, psi - kPi);
            put_cubic(T + 4 * (r ? kExitPhi0B : kExitPhi0), i, phi0);
        }
        put_cubic(T + 4 * kExitIc, i, Ic);
        put_pair<true>(T + 4 * kExitRange, i, B::template sweep<float>(fminf(1.0f / (sv.rule.disk_inner * 0.97f), Rt.u2), Rt, beta),
                       B::template sweep<float>(fminf(1.0f / (sv.rule.disk_outer * 1.03f), Rt.u2), Rt, beta));
        put_pair<false>(T + 4 * kExitU2, i, Rt.u2, 0.f);
    }
}

// The learned surrogate's tables of a batch of views in one launch on the tensor cores: every
// view's exit table (the escaping half per branch of the rule's exit, the captured half) and
// crossing table, as 128-row tiles of network queries. A block is one warpgroup with its own TMEM
// accumulator; it stages the network once (tc::load_net, tc::load_l1) and then takes tiles until
// the batch is done. Each thread forms its row's query (for an escaping exit point, from the closed
// form at the point), the tile runs through tc::mlp_tile_l1f, and each thread writes its row's
// results into the table entries that hold them (a point enters four cubic windows and two
// linear pairs). A completion wait that runs out makes the block write NaN for its tile, set
// *status and stop.
__global__ void __launch_bounds__(128, 4) k_tables(const __grid_constant__ TabBatch B, const float* __restrict__ P,
                                                   int* __restrict__ status) {
    extern __shared__ __align__(16) unsigned char smem_raw[];
    tc::Net& N = *reinterpret_cast<tc::Net*>(smem_raw);
    tc::L1& l1 = *reinterpret_cast<tc::L1*>(smem_raw + sizeof(tc::Net));
    tc::Tile& T = *reinterpret_cast<tc::Tile*>(smem_raw + sizeof(tc::Net) + sizeof(tc::L1));
    __shared__ uint32_t tmem_slot;
    __shared__ int fail;
    tc::load_net(N, P, false, 0.f);
    tc::load_l1(l1, P);
    if (threadIdx.x == 0) {
        tc::mbar_init(tc::smem_u32(&T.mbar), 1);
        fail = 0;
    }
    if (threadIdx.x < 32) tc::tmem_alloc(tc::smem_u32(&tmem_slot), tc::kTmemCols);
    tc::fence_smem_async();
    tc::fence_before();
    __syncthreads();
    tc::fence_after();
    const uint32_t tmem = tmem_slot;
    uint32_t phase = 0;
    const Norm& nm = B.norm;
    const int row = int(threadIdx.x);
    constexpr float kPi = 3.14159265358979f;
    const float hs = 2.0f / float(kCrossNs - 1);
    for (int tile = blockIdx.x; tile < B.ntiles; tile += gridDim.x) {
        int v = 0;
        while (v + 1 < B.nviews && B.v[v + 1].tile0 <= tile) ++v;
        const TabView& V = B.v[v];
        const int t = tile - V.tile0;
        const int nesc = kTabTilesExit * (V.tol ? 2 : 1);
        // kind 0: an escaping exit point (branch r); 1: a captured exit point; 2: a crossing cell corner
        const int kind = t < nesc ? 0 : (t < nesc + kTabTilesExit ? 1 : 2);
        const int r = kind == 0 ? t / kTabTilesExit : 0;
        int i = 0, jj = 0;
        float x2, sigma = 1.0f;  // the capture flag is trained at sigma = 1
        float b = 0.f, beta = 0.f, Ic = 0.f, Ie = 0.f, ue = 0.f;
        orbit::Roots<float> Rt{};
        if (kind == 0) {
            i = (t - r * kTabTilesExit) * 128 + row;
            x2 = fmaf(float(i), B.tab_h[1], B.tab_lo[1]);
            beta = fmaxf(nm.t_eps * expm1f(x2 / nm.t_scale), 1e-7f);
            b = kSqrt27f * (1.0f + beta);
            Rt = orbit::roots<float, 4>(beta);
            ue = !V.tol ? nm.ue : (r == 0 ? fminf(V.u_esc_min, Rt.u2) : orbit::exit_u_tol<float>(b, V.esc_tol, 1.0f, Rt.u2));
            sigma = orbit::sigma_exit<float>(ue, Rt);
            using Bl = orbit::Baseline<true>;
            Ic = Bl::template sweep<float>(V.uc, Rt, beta);
            Ie = Bl::template sweep<float>(ue, Rt, beta);
        } else if (kind == 1) {
            i = (t - nesc) * 128 + row;
            x2 = fmaf(float(i), B.tab_h[0], B.tab_lo[0]);
        } else {
            const int c = (t - nesc - kTabTilesExit) * 128 + row;
            i = c / kCrossNs;
            jj = c - i * kCrossNs;
            x2 = fmaf(float(i), B.cx_h, B.tab_lo[1]);
            sigma = fmaf(float(jj), hs, -1.0f);
        }
        float2 o;
        const bool ok = tc::mlp_tile_l1f(N, l1, T, tmem, row, 1, phase, make_float4(V.x1, x2, sigma, 0.f), o);
        if (!ok) {
            fail = 1;
            o = make_float2(__int_as_float(0x7fc00000), __int_as_float(0x7fc00000));
        }
        if (kind == 0) {
            float* E = reinterpret_cast<float*>(V.exit_table);
            const float phi0 = Ic + Ie + o.x * nm.y_scale;
            const float psi = escape_angle(phi0, ue, Rt, b, V.two_over_r3);
            put_cubic(E + 4 * (r ? kExitPsiB : kExitPsi), i, psi - kPi);
            put_cubic(E + 4 * (r ? kExitPhi0B : kExitPhi0), i, phi0);
            if (r == 0) {
                using Bl = orbit::Baseline<true>;
                put_cubic(E + 4 * kExitIc, i, Ic);
                put_pair<true>(E + 4 * kExitRange, i,
                               Bl::template sweep<float>(fminf(1.0f / (V.disk_inner * 0.97f), Rt.u2), Rt, beta),
                               Bl::template sweep<float>(fminf(1.0f / (V.disk_outer * 1.03f), Rt.u2), Rt, beta));
            }
            if (r == (V.tol && b > V.b_kink ? 1 : 0)) put_pair<false>(E + 4 * kExitU2, i, Rt.u2, o.y);
        } else if (kind == 1) {
            put_pair<true>(reinterpret_cast<float*>(V.exit_table), i, o.x, o.y);
        } else {
            constexpr int W = kCrossNs - 1;  // cells per row
            float* c = reinterpret_cast<float*>(V.cross_table);
            const float y = o.x;
            if (i < kCrossNx - 1 && jj < W) c[4 * (i * W + jj) + 0] = y;
            if (i < kCrossNx - 1 && jj > 0) c[4 * (i * W + jj - 1) + 1] = y;
            if (i > 0 && jj < W) c[4 * ((i - 1) * W + jj) + 2] = y;
            if (i > 0 && jj > 0) c[4 * ((i - 1) * W + jj - 1) + 3] = y;
        }
        __syncthreads();
        if (fail) break;
    }
    if (fail && threadIdx.x == 0) atomicExch(status, 1);
    tc::fence_before();
    __syncthreads();
    if (threadIdx.x < 32) {
        tc::fence_after();
        tc::tmem_dealloc(tmem, tc::kTmemCols);
    }
}

// The crossing query's y from the view's table: bilinear in (x2, sigma).
__device__ __forceinline__ float cross_from_table(const SurrView& sv, float x2, float sigma) {
    constexpr int W = kCrossNs - 1;
    const float u = (x2 - sv.tab_lo[1]) * sv.cx_inv_h;
    const float v = (sigma + 1.0f) * (0.5f * float(kCrossNs - 1));
    const int i = min(max(int(floorf(u)), 0), kCrossNx - 2), j = min(max(int(floorf(v)), 0), kCrossNs - 2);
    const float a = u - float(i), b = v - float(j);
    const float4 q = __ldg(sv.cross_table + i * W + j);
    const float lo = fmaf(b, q.y - q.x, q.x), hi = fmaf(b, q.w - q.z, q.z);
    return fmaf(a, hi - lo, lo);
}


// Lagrange weights of the cubic through the entry's four points (nodes 0 .. 3) at tc in [0, 3].
__device__ __forceinline__ float4 cubic_weights(float tc) {
    const float a = tc, b = tc - 1.0f, c = tc - 2.0f, d = tc - 3.0f;
    const float ab = a * b, cd = c * d;
    return make_float4(-(1.0f / 6.0f) * b * cd, 0.5f * a * cd, -0.5f * ab * d, (1.0f / 6.0f) * ab * c);
}
__device__ __forceinline__ float cubic(const float4 f, const float4 L) {
    return fmaf(f.x, L.x, fmaf(f.y, L.y, fmaf(f.z, L.z, f.w * L.w)));
}

// The captured half's capture logit at x2 (linear between the two points of entry m).
__device__ __forceinline__ float capture_logit(const SurrView& sv, float x2) {
    const float u = (x2 - sv.tab_lo[0]) * sv.tab_inv_h[0];
    const int i = min(max(int(floorf(u)), 0), kExitTableN - 2);
    const float4 e = __ldg(sv.exit_table + i);
    return fmaf(u - float(i), e.w - e.y, e.y);
}

template <bool kTol, bool kNet>
__global__ void __launch_bounds__(32 * kInferWarps, surr_blocks_per_sm(kNet)) k_surrogate(const __grid_constant__ SurrView sv,
                                                                WorkQueue* q, int* __restrict__ fb_list) {
    extern __shared__ __align__(16) unsigned char smem_raw[];
    InferSmem& S = *reinterpret_cast<InferSmem*>(smem_raw);
    const DevView& w = sv.view;
    const Rule& R = sv.rule;
    const Norm& nm = sv.norm;
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    RayStage& G = S.st[warp];
    int* task = S.task[warp];
    float* tu = S.tu[warp];
    float* tphi = S.tphi[warp];
    constexpr float kPi = 3.14159265358979f;
    const float beta_band = nm.band / kSqrt27f;
    const float uc = sv.uc;
    // records go out as two 32-byte stores when the view's buffer allows it (records are 64 B,
    // so every record is then 32-byte aligned); the interface guarantees 16 bytes
    const bool out32 = (reinterpret_cast<uintptr_t>(w.out) & 31u) == 0;
    const bool thin = R.disk_mode == BHR_DISK_THIN;
    const float4* E = sv.exit_table;
    uint32_t n_surr = 0, n_dis = 0;
    // a warp claims four 32-ray chunks per atomic on the view's counter: one claim per chunk made
    // the counter's atomics a serial point (65,000 a view; two per claim measured 6% faster, four
    // another 0.5-2%, with the grid's four blocks per SM)
    constexpr int kClaim = 4;
    unsigned long long claim = 0;
    int left = 0;
    for (;;) {
        if (left == 0) {
            if (lane == 0) claim = atomicAdd(&q->next_chunk, (unsigned long long)kClaim);
            claim = __shfl_sync(0xffffffffu, claim, 0);
            left = kClaim;
        }
        const unsigned long long chunk = claim + (unsigned long long)(kClaim - left);
        --left;
        const int64_t base = (int64_t)chunk * 32;
        if (base >= w.nrays) break;
        const int ray = int(base + lane);
        const bool valid = ray < w.nrays;
        // rays of the band march (k_band_list) are neither answered nor sent to the fallback list
        const bool pre = sv.band_mask != nullptr && ((__ldg(sv.band_mask + chunk) >> lane) & 1u) != 0u;
        // ---- phase 1: per ray
        int ncand = 0;
        // what only this lane's record needs stays in registers through phase 2
        float o_psi = 0.f, o_minr = 0.f, o_baxis = 0.f, o_b = 0.f;
        V3<float> o_e2{0.f, 0.f, 0.f};
        uint32_t o_info = 0;
        {
            bool sur = valid && !pre;
            // row and column: the quotient from a float reciprocal of the width, then corrected by
            // one either way (exact for views up to 2^22 rows; 2% of the step faster than the
            // integer division)
            int j = __float2int_rz(float(ray) * (1.0f / float(w.width)));
            j -= (j * w.width > ray) ? 1 : 0;
            j += ((j + 1) * w.width <= ray) ? 1 : 0;
            j = valid ? j : 0;
            const int i = valid ? ray - j * w.width : 0;
            // the pixel's direction, its angle from the radial direction e1 and b = r sin(angle) /
            // sqrt(1 - 2 / r): the reference's h / |v_inf| for the initial velocity of
            // geodesic.glsl:27-34 (whose radial part the lapse scales), without forming that
            // velocity; its tangential part, and so the orbital plane, is d's. The direction of
            // blackhole.frag:68-72 is the camera basis times (cx, cy, -1), normalised, with cx and
            // cy affine in the pixel: one normalisation of an affine map of (i, j) about the
            // image's centre (within 1.3e-7 rad of the FP64 direction at 1080p; the shader's two
            // divisions and two normalisations were 5% of the step)
            V3<float> d;
            {
                const float fi = float(i - sv.i_mid), fj = float(j - sv.j_mid);
                d = {fmaf(fi, sv.dir_i[0], fmaf(fj, sv.dir_j[0], sv.dir_0[0])),
                     fmaf(fi, sv.dir_i[1], fmaf(fj, sv.dir_j[1], sv.dir_0[1])),
                     fmaf(fi, sv.dir_i[2], fmaf(fj, sv.dir_j[2], sv.dir_0[2]))};
                const float dn = rsqrtf(dot3(d, d));
                d = {d.x * dn, d.y * dn, d.z * dn};
            }
            const V3<float> e1{w.rhat[0], w.rhat[1], w.rhat[2]};
            const V3<float> cx{e1.y * d.z - e1.z * d.y, e1.z * d.x - e1.x * d.z, e1.x * d.y - e1.y * d.x};
            float b = sv.b_scale * orbit::FM<float>::sqrt(dot3(cx, cx));
            float beta = b * (1.0f / kSqrt27f) - 1.0f;
            if (sur && fabsf(beta) < 0.02f) {  // near the photon sphere: impact parameter in FP64
                const double bd = impact_parameter_fp64(w, sv.fc, i, j);
                beta = float(bd * (1.0 / kSqrt27d) - 1.0);
                b = float(bd);
            }
            // captured orbits (b < sqrt(27)) are answered too: the network gives their capture flag,
            // the closed form their crossings (no turning point, no learned residual)
            const bool cap = beta < 0.f;
            const float ve = dot3(d, e1);  // ingoing at the camera: ve < 0
            sur = sur && ve < 0.f && w.rcam >= nm.rc_lo && w.rcam <= nm.rc_hi && b <= nm.b_max &&
                  fabsf(beta) >= beta_band;
            // orbital plane: e1 along the camera, e2 along the tangential part of the direction
            V3<float> e2{d.x - ve * e1.x, d.y - ve * e1.y, d.z - ve * e1.z};
            const float e2n = dot3(e2, e2);
            sur = sur && e2n > 1e-12f;
            const float e2i = rsqrtf(fmaxf(e2n, 1e-30f));
            e2 = {e2.x * e2i, e2.y * e2i, e2.z * e2i};
            const float tb = __logf(1.0f + fabsf(beta) * (1.0f / nm.t_eps));  // 1 + |beta|/eps >= 1.19 here
            const float x2 = (beta < 0.f ? -tb : tb) * nm.t_scale;
            // stage slots: escaping orbit: psi, minr, Ic = angle camera -> turning point; captured orbit:
            // u1, A, k^2, K, Ic = F(camera); phi0 = angle camera -> exit (or -> horizon)
            float s0 = 0.f, s1 = 0.f, s2 = 0.f, s3 = 0.f, Ic = 0.f, phi0 = 0.f, psi = 0.f, minr = 0.f;
            float Ilo = 1.f, Ihi = 0.f;  // angle range of the disk's crossings (from the turning point / camera)
            float gx = 0.f;
            int m = 0, jc = 0;
            if (!cap) {
                sur = sur && x2 < sv.x2_lim;  // clear of the camera's tangential ray
                // the exit table: pair entry m and cubic entry jc around the ray's x2
                gx = (x2 - sv.tab_lo[1]) * sv.tab_inv_h[1];
                m = min(max(int(floorf(gx)), 0), kExitTableN - 2);
                jc = min(max(m - 1, 0), kExitTableN - 4);
                const float4 L = cubic_weights(gx - float(jc));
                const float4 pu = __ldg(E + kExitU2 + m);
                const float t = gx - float(m);
                const float u2 = fmaf(t, pu.y - pu.x, pu.x);
                sur = sur && uc < u2 * 0.9999f;
                if (kNet && sur && fmaf(t, pu.w - pu.z, pu.z) > 0.f) {  // the learned capture flag disagrees with
                    sur = false;                                         // b vs sqrt(27): the integrator decides
                    ++n_dis;
                }
                const bool br = kTol && b > sv.b_kink;  // the tolerance escape's branch
                // the turning point's angle and the disk's range are loaded with the others, so
                // that the five loads' latencies overlap (they are used only when the ray has
                // plane crossings)
                const float4 ei = __ldg(E + kExitIc + jc);
                const float4 rg = __ldg(E + kExitRange + m);
                psi = cubic(__ldg(E + (br ? kExitPsiB : kExitPsi) + jc), L);
                phi0 = cubic(__ldg(E + (br ? kExitPhi0B : kExitPhi0) + jc), L);
                minr = orbit::FM<float>::rcp(u2);
                Ic = cubic(ei, L);
                if (thin) {
                    Ilo = fmaf(t, rg.z - rg.x, rg.x);
                    Ihi = fmaf(t, rg.w - rg.y, rg.y);
                }
            } else {
                if (kNet && sur && !(capture_logit(sv, x2) > 0.f)) {
                    sur = false;
                    ++n_dis;
                }
                if (sur) {
                    const CapStage cs = cap_stage(beta, uc, R.capture_r, R.disk_inner, R.disk_outer, thin);
                    Ic = cs.Ic, phi0 = cs.phi0, Ilo = cs.Ilo, Ihi = cs.Ihi;
                    s0 = cs.u1, s1 = cs.A, s2 = cs.k2, s3 = cs.K;
                }
            }
            // disk-plane crossings: y(phi) = 0 at phi_k = phi_n + k pi
            float phin = orbit::atan_ratio(-e1.y, e2.y);  // the nodal line's angle, taken in [0, pi)
            if (phin < 0.f) phin += kPi;
            if (phin >= kPi) phin -= kPi;
            sur = sur && (fabsf(e1.y) + fabsf(e2.y)) > 1e-6f;
            int nplane = 0;
            uint32_t cw = 0;
            if (sur) {
                // crossings k = 0, 1, ... with phin + k pi < phi0 (at most 16)
                if (phi0 > phin) nplane = min(int(ceilf((phi0 - phin) * (1.0f / kPi))), 16);
                // crossing k lies in [0.97 r_in, 1.03 r_out] iff its angle from the turning point,
                // |phi_k - Ic|, lies between the sweeps to those radii (or to the turning point,
                // where the orbit stays outside them): [Ilo, Ihi] from the exit table
#pragma unroll 1
                for (int k = 0; k < nplane && ncand < kMaxCand; ++k) {
                    const float phk = phin + float(k) * kPi;
                    const bool leg = !cap && phk > Ic;
                    const float tg = cap ? phk : (leg ? phk - Ic : Ic - phk);
                    if (tg >= Ilo && tg <= Ihi) {
                        cw |= (uint32_t(k) | (leg ? 16u : 0u)) << (11 + 5 * ncand);
                        ++ncand;
                    }
                }
            }
            // phase 2 reads the stage of rays with candidates only
            if (__any_sync(0xffffffffu, ncand > 0)) {
                G.s0[lane] = s0;
                G.s1[lane] = s1;
                G.s2[lane] = s2;
                G.s3[lane] = s3;
                G.ic[lane] = Ic;
                G.phin[lane] = phin;
                G.x2[lane] = x2;
                G.beta[lane] = beta;
                // the crossings' direction from the hole: phi_k = phin + k pi gives cos(phi_k) e1 +
                // sin(phi_k) e2 = (-1)^k n, n along (e2.y e1 - e1.y e2) with the sign that makes
                // sin(phin) >= 0 (phin in [0, pi)); no trigonometry per crossing
                const float sn = e1.y < 0.f ? 1.f : (e1.y > 0.f ? -1.f : (e2.y >= 0.f ? 1.f : -1.f));
                G.nx[lane] = sn * (e2.y * e1.x - e1.y * e2.x);
                G.nz[lane] = sn * (e2.y * e1.z - e1.y * e2.z);
                G.b[lane] = b;
            }
            o_info = uint32_t(ncand) | (sur ? 4u : 0u) | (uint32_t(min(nplane, 255)) << 3) | cw | (cap ? kCapBit : 0u);
            G.info[lane] = o_info;
            o_psi = psi;
            o_minr = minr;
            // impactParameterAboutAxis: -dot(cross(cam, dir), +Y) / sqrt(max(1 - 2/r, 1e-6))
            o_baxis = -(w.cam[2] * d.x - d.z * w.cam[0]) * w.baxis_scale;
            o_b = b;
            o_e2 = e2;
        }
        // ---- phase 2: crossing candidates, compacted over the lanes
        int off = ncand;
#pragma unroll
        for (int d = 1; d < 32; d <<= 1) {
            const int y = __shfl_up_sync(0xffffffffu, off, d);
            if (lane >= d) off += y;
        }
        const int total = __shfl_sync(0xffffffffu, off, 31);
        off -= ncand;
        for (int c = 0; c < ncand; ++c) task[off + c] = (lane << 2) | c;
        __syncwarp();
#pragma unroll 1
        for (int t = lane; t < total; t += 32) {
            const int own = task[t] >> 2, c = task[t] & 3;
            const uint32_t info = G.info[own];
            const uint32_t kl = (info >> (11 + 5 * c)) & 31u;
            const float phk = G.phin[own] + float(kl & 15u) * kPi;
            const float Ic = G.ic[own];
            float us;
            if (!(info & kCapBit)) {
                const float beta = G.beta[own];
                const orbit::Roots<float> Rt = orbit::roots<float, 4>(fmaxf(beta, 1e-7f));
                const bool leg = (kl & 16u) != 0;
                // three Newton steps: within 2e-6 of the crossing's u (relative) for every crossing
                // of the disk's radii (the fourth step measured 1% of the step for nothing visible)
                const float u = orbit::invert_sweep_v<float, 3, kNet>(leg ? phk - Ic : Ic - phk, Rt, beta);
                us = u;
                if (kNet) {  // the network's residual from the view's crossing table, applied along the orbit
                    const float sg =
                        leg ? orbit::FM<float>::sqrt(fmaxf((Rt.u2 - u) * orbit::FM<float>::rcp(Rt.u2), 0.f))
                            : -orbit::FM<float>::sqrt(fmaxf((Rt.u2 - u) * orbit::FM<float>::rcp(Rt.u2 - uc), 0.f));
                    const float dphi = cross_from_table(sv, G.x2[own], sg) * nm.y_scale;
                    const float sPu = orbit::dudphi<float>(u, Rt);
                    us = leg ? u + dphi * sPu : u - dphi * sPu;
                }
            } else {
                us = cap_invert(G.s0[own], G.s1[own], G.s2[own], G.s3[own], G.b[own], Ic, phk, uc, R.capture_r,
                                R.disk_inner, R.disk_outer);
            }
            const float rs = orbit::FM<float>::rcp(us);
            float rr = -1.f, ph = 0.f;
            if (rs >= R.disk_inner && rs <= R.disk_outer) {
                const float sk = (kl & 1u) ? -1.f : 1.f;  // the nodal line's far end for odd k
                ph = orbit::atan2_fast(sk * G.nz[own], sk * G.nx[own]);
                rr = rs;
            }
            tu[t] = rr;
            tphi[t] = ph;
        }
        __syncwarp();
        // ---- phase 3: records (per ray)
        {
            const uint32_t info = o_info;
            const bool sur = (info & 4u) != 0;
            const bool cap = (info & kCapBit) != 0;
            if (valid && !sur && !pre) fb_list[warp_append_ull(&q->fb_count)] = ray;
            if (sur) {
                ++n_surr;
                // captured: no direction (as TraceResult::dir), closest approach = the capture radius
                V3<float> d{0.f, 0.f, 0.f};
                float min_r = R.capture_r;
                uint32_t status = BHR_STATUS_CAPTURED;
                if (!cap) {  // the escape direction cos(psi) e1 + sin(psi) e2, psi = pi + the table's angle
                    float sp, cp;
                    sincos_rr(o_psi, &sp, &cp);
                    d = {-(cp * w.rhat[0] + sp * o_e2.x), -(cp * w.rhat[1] + sp * o_e2.y),
                         -(cp * w.rhat[2] + sp * o_e2.z)};
                    min_r = o_minr;
                    status = BHR_STATUS_ESCAPED;
                }
                // crossings inside [disk_inner, disk_outer], in march order
                const int nc = int(info & 3u);
                float cr[3] = {0.f, 0.f, 0.f}, cph[3] = {0.f, 0.f, 0.f};
                int nrec = 0;
#pragma unroll
                for (int c = 0; c < kMaxCand; ++c) {
                    if (c < nc) {
                        const float rr = tu[off + c];
                        if (rr > 0.f) {
                            const float pp = tphi[off + c];
                            cr[0] = nrec == 0 ? rr : cr[0];
                            cph[0] = nrec == 0 ? pp : cph[0];
                            cr[1] = nrec == 1 ? rr : cr[1];
                            cph[1] = nrec == 1 ? pp : cph[1];
                            cr[2] = nrec == 2 ? rr : cr[2];
                            cph[2] = nrec == 2 ? pp : cph[2];
                            ++nrec;
                        }
                    }
                }
                const uint32_t nplane = (info >> 3) & 0xffu;
                const uint32_t w0 = status | (uint32_t(nrec) << 8) | (uint32_t(BHR_FLAG_SURROGATE) << 16) | (nplane << 24);
                if (out32) {  // two 32-byte stores: each covers whole sectors
                    st_global_v8(w.out + ray, w0, 0u, __float_as_uint(d.x), __float_as_uint(d.y),
                                 __float_as_uint(d.z), __float_as_uint(min_r), 0u, 0u);
                    st_global_v8(reinterpret_cast<const char*>(w.out + ray) + 32, __float_as_uint(o_baxis),
                                 __float_as_uint(o_b), __float_as_uint(cr[0]), __float_as_uint(cr[1]),
                                 __float_as_uint(cr[2]), __float_as_uint(cph[0]), __float_as_uint(cph[1]),
                                 __float_as_uint(cph[2]));
                } else {
                    float4* p = reinterpret_cast<float4*>(w.out + ray);
                    p[0] = make_float4(__uint_as_float(w0), __uint_as_float(0u), d.x, d.y);
                    p[1] = make_float4(d.z, min_r, 0.f, 0.f);
                    p[2] = make_float4(o_baxis, o_b, cr[0], cr[1]);
                    p[3] = make_float4(cr[2], cph[0], cph[1], cph[2]);
                }
            }
        }
        __syncwarp();
    }
    for (int o = 16; o > 0; o >>= 1) {
        n_surr += __shfl_xor_sync(0xffffffffu, n_surr, o);
        n_dis += __shfl_xor_sync(0xffffffffu, n_dis, o);
    }
    if (lane == 0) {
        atomicAdd(&q->surr_rays, (unsigned long long)n_surr);
        if (n_dis) atomicAdd(&q->capture_disagree, (unsigned long long)n_dis);
    }
}

}  // namespace

int train_smem_bytes() { return int(sizeof(TrainSmem)); }


cudaError_t launch_surrogate_trace(const SurrView& sv, WorkQueue* q, int* fb_list, int grid, bool net,
                                   cudaStream_t st) {
    const int smem = int(sizeof(InferSmem));
    const bool tol = sv.rule.term_mode != BHR_TERM_CONFIG;
    using K = void (*)(SurrView, WorkQueue*, int*);
    const K kern = tol ? (net ? K(k_surrogate<true, true>) : K(k_surrogate<true, false>))
                       : (net ? K(k_surrogate<false, true>) : K(k_surrogate<false, false>));
    // the driver's own split of the SM's memory: the blocks need at most 90 KB of shared memory, and
    // the rest serves as L1 for the views' tables (the largest carveout left 28 KB of L1, a 20%
    // hit rate on the table loads, and was 2% slower)
    const cudaError_t e = prefer_max_smem((const void*)kern, smem, false);
    if (e != cudaSuccess) return e;
    kern<<<grid, 32 * kInferWarps, smem, st>>>(sv, q, fb_list);
    return cudaGetLastError();
}

cudaError_t launch_orbit_data(uint64_t seed, int64_t n_orbits, int k_per_orbit, const Norm& nrm, double step_frac,
                              TrainSample* X, int8_t* lab, unsigned long long* stats, int grid, cudaStream_t st) {
    if (k_per_orbit < 2 || k_per_orbit > kMaxK) return cudaErrorInvalidValue;
    k_orbit_data<<<grid, 128, 0, st>>>(seed, n_orbits, k_per_orbit, nrm, step_frac, X, lab, stats);
    return cudaGetLastError();
}

cudaError_t launch_train_step(const float* params, const TrainSample* X, const int8_t* lab, int64_t n_samples,
                              const int64_t* idx, int batch, uint64_t seed, float w_u, float w_c, float* grads,
                              float* loss, int grid, cudaStream_t st) {
    const int smem = train_smem_bytes();
    const cudaError_t e = prefer_max_smem((const void*)k_train_step, smem, false);
    if (e != cudaSuccess) return e;
    k_train_step<<<grid, 32 * kTrainWarps, smem, st>>>(params, X, lab, n_samples, idx, batch, seed, w_u, w_c, grads,
                                                        loss);
    return cudaGetLastError();
}

cudaError_t launch_adam(float* params, float* grads, float* m, float* v, int step, float lr, float beta1,
                        float beta2, float eps, cudaStream_t st) {
    k_adam<<<(kNParams + 255) / 256, 256, 0, st>>>(params, grads, m, v, step, lr, beta1, beta2, eps);
    return cudaGetLastError();
}

cudaError_t launch_exit_table_cf(const SurrView& sv, float4* table, cudaStream_t st) {
    const int grid = (kExitTableN + 255) / 256;  // one point per thread
    const bool tol = sv.rule.term_mode != BHR_TERM_CONFIG;
    const cudaError_t e =
        prefer_max_smem(tol ? (const void*)k_exit_table_cf<true> : (const void*)k_exit_table_cf<false>, 0, true);
    if (e != cudaSuccess) return e;
    if (tol) k_exit_table_cf<true><<<grid, 256, 0, st>>>(sv, table);
    else k_exit_table_cf<false><<<grid, 256, 0, st>>>(sv, table);
    return cudaGetLastError();
}

cudaError_t launch_band_list(const BandBatch& b, cudaStream_t st) {
    if (b.total_rows <= 0) return cudaSuccess;
    const cudaError_t e = prefer_max_smem((const void*)k_band_list, 0, true);
    if (e != cudaSuccess) return e;
    k_band_list<<<(b.total_rows + 3) / 4, 128, 0, st>>>(b);
    return cudaGetLastError();
}

bool band_rows(const bhr_view& v, const Fp64Cam& fc, double b_lo, double b_hi, BandRows* q) {
    // sin of the angle from the hole for impact parameter b: b / b_scale
    const double s_hi = b_hi / fc.b_scale_d, s_lo = std::max(b_lo, 0.0) / fc.b_scale_d;
    if (!(s_hi < 1.0) || !(s_lo < s_hi)) return false;
    const double R[3] = {v.cam_basis[0], v.cam_basis[1], v.cam_basis[2]};
    const double U[3] = {v.cam_basis[3], v.cam_basis[4], v.cam_basis[5]};
    const double B[3] = {v.cam_basis[6], v.cam_basis[7], v.cam_basis[8]};
    const double* rh = fc.rhat_d;
    auto dot = [](const double* x, const double* y) { return x[0] * y[0] + x[1] * y[1] + x[2] * y[2]; };
    const double bn = std::sqrt(dot(B, B));
    if (!(bn > 0.0)) return false;
    // the view axis is -B; the hole is at -rhat
    const double theta = std::acos(std::min(1.0, std::max(-1.0, dot(B, rh) / bn)));
    if (!(theta + std::asin(s_hi) < 85.0 * 3.14159265358979323846 / 180.0)) return false;
    q->c_out = float(1.0 - s_hi * s_hi);
    q->c_in = float(1.0 - s_lo * s_lo);
    q->a = float(dot(rh, R));
    q->rhU = float(dot(rh, U));
    q->rhB = float(dot(rh, B));
    q->RR = float(dot(R, R));
    q->RU = float(dot(R, U));
    q->RB = float(dot(R, B));
    q->UU = float(dot(U, U));
    q->UB = float(dot(U, B));
    q->BB = float(dot(B, B));
    return true;
}

cudaError_t launch_tables(const TabBatch& b, const float* params, int* status, int grid, cudaStream_t st) {
    const int smem = int(sizeof(tc::Net) + sizeof(tc::L1) + sizeof(tc::Tile));
    const cudaError_t e = prefer_max_smem((const void*)k_tables, smem, true);
    if (e != cudaSuccess) return e;
    k_tables<<<std::max(1, std::min(grid, b.ntiles)), 128, smem, st>>>(b, params, status);
    return cudaGetLastError();
}

cudaError_t launch_mlp_infer(const float* params, const float4* q, float2* out, int n, int* status, int grid,
                             cudaStream_t st, long long wait_cycles, bool withhold) {
    tc::TileCtl ctl;
    if (wait_cycles > 0) ctl.wait_cycles = wait_cycles;
    ctl.withhold = withhold;
    k_mlp_infer<<<grid, 128, sizeof(tc::Net) + sizeof(tc::L1) + sizeof(tc::Tile), st>>>(params, q, out, n, status, ctl);
    return cudaGetLastError();
}

}  // namespace surr
}  // namespace bhr
