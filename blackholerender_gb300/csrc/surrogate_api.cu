// C ABI of the learned orbit surrogate (include/bhr.h, "surrogate" section): creation, training
// data from the integrator, training, parameter access, the gradient check hook, save/load, and
// the surrogate-plus-fallback trace.
#include <cuda_runtime.h>

#include <algorithm>
#include <array>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <new>
#include <string>
#include <vector>

#include "bhr.h"
#include "host_views.h"
#include "kernels.cuh"
#include "surrogate.cuh"

using bhr::surr::kNParams;

// One trace pipeline: its work memory, streams and events. Lane 0 serves bhr_surrogate_trace and
// plans; bhr_surrogate_trace_host alternates lanes 0 and 1, whose traces overlap on the GPU, so
// nothing a trace writes is shared between lanes.
struct SurrLane {
    // work queues of a trace of n views: [2v] view v's pass, [2v+1] its own fallback march,
    // [2n] the fallback march of all views; then the band march's: [2n+1+2v] view v's band list
    // count, [4n+1] the band march itself
    bhr::WorkQueue* q = nullptr;
    int64_t nq = 0;
    int* fb = nullptr;  // fallback ray lists, one per view, one after the other
    int64_t fb_cap = 0;
    uint32_t* mask = nullptr;  // band masks, one bit per ray, per view ceil(rays / 32) words
    int64_t mask_cap = 0;
    int* band = nullptr;  // band lists, kBandCap rays per view
    int64_t band_cap = 0;
    float4* etab = nullptr;  // the views' exit tables, [view][kExitTabEntries]
    int64_t etab_cap = 0;
    float4* ctab = nullptr;  // the views' crossing tables, [view][kCrossCells]
    int64_t ctab_cap = 0;
    // the views' passes alternate between side[0] and side[1] (fork / join on the caller's
    // stream), so each launch's last wave overlaps the next view's first; side[2] finds and
    // marches the band rays beside them
    cudaStream_t side[3] = {nullptr, nullptr, nullptr};
    cudaEvent_t start = nullptr, fork = nullptr, band_ready = nullptr;
    cudaEvent_t join[3] = {nullptr, nullptr, nullptr};
    cudaEvent_t ev[3] = {nullptr, nullptr, nullptr};  // timing: start, passes done, fallback done
};

struct bhr_surrogate {
    int device = 0;
    int sms = 0;
    bhr::surr::Norm norm{};
    float* params = nullptr;  // FP32 master weights (device)
    float* grads = nullptr;
    float* adam_m = nullptr;
    float* adam_v = nullptr;
    int adam_step = 0;
    bhr::surr::TrainSample* X = nullptr;  // training samples (device)
    int8_t* lab = nullptr;
    int64_t n_samples = 0;
    unsigned long long* stats = nullptr;  // data generation counters (device, 4)
    int* tab_status = nullptr;  // per lane, set on the device when a table build's tensor-core wait ran out
    float* loss = nullptr;                // per-step loss sums (device, 3 * loss_cap)
    int loss_cap = 0;
    bool use_network = true;  // false: the non-learned variant (tables from the converged closed form)
    SurrLane lane[2];
    uint64_t work_gen = 0;  // bumped whenever a trace reallocates lane 0's work memory (plans hold pointers into it)
    unsigned long long last[4] = {0, 0, 0, 0};
    // the last trace: its stream, lane, views and network rows
    cudaStream_t last_stream = nullptr;
    int last_lane = 0;
    int last_nviews = 0;
    uint64_t last_rows = 0;
    bool have_last = false;
    bool last_from_plan = false;  // the last trace was a graph replay (its events do not time)
    // bhr_surrogate_trace_host: device staging and two streams
    bhr_hit* staging = nullptr;
    int64_t staging_rays = 0;
    cudaStream_t hs[2] = {nullptr, nullptr};
};

namespace {

// The b at which the tolerance escape's exit moves from rEscMin (u_esc_min) to u_tol(b): the root
// of 0.75 b'^3 u^4 = tol at u = u_esc_min, b' = b / sqrt(1 + 2 b^2 u^3). The estimate rises with b
// (its log-derivative is 3 / (b (1 + 2 b^2 u^3)) > 0), so bisection finds it; below sqrt(27)
// or above 1e4 it is clamped there (one branch serves every escaping ray).
float tolerance_kink(float tol, float u_esc_min) {
    const double u = u_esc_min, t = tol;
    auto est = [&](double b) { return 0.75 * std::pow(b / std::sqrt(1.0 + 2.0 * b * b * u * u * u), 3.0) * u * u * u * u; };
    double lo = 5.196152422706632, hi = 1e4;
    if (est(lo) >= t) return float(lo);
    if (est(hi) < t) return float(hi);
    for (int k = 0; k < 200; ++k) {
        const double mid = 0.5 * (lo + hi);
        (est(mid) < t ? lo : hi) = mid;
    }
    return float(0.5 * (lo + hi));
}

int fail(int code, const std::string& msg) {
    bhr::set_last_error(msg);
    return code;
}
int cfail(cudaError_t e, const char* what) { return fail(BHR_ERR_CUDA, std::string(what) + ": " + cudaGetErrorString(e)); }

struct DevGuard {
    int prev = 0;
    explicit DevGuard(int dev) {
        cudaGetDevice(&prev);
        cudaSetDevice(dev);
    }
    ~DevGuard() { cudaSetDevice(prev); }
};

template <class T>
cudaError_t grow(T** p, int64_t* cap, int64_t need) {
    if (need <= *cap) return cudaSuccess;
    if (*p) cudaFree(*p);
    *p = nullptr;
    *cap = 0;
    cudaError_t e = cudaMalloc(p, sizeof(T) * size_t(need));
    if (e == cudaSuccess) *cap = need;
    return e;
}

// Glorot-uniform initialisation, deterministic from the seed (host side).
void init_params(std::vector<float>& P, uint64_t seed) {
    uint64_t s = seed * 0x9E3779B97F4A7C15ull + 1;
    auto unif = [&]() {
        s ^= s << 13;
        s ^= s >> 7;
        s ^= s << 17;
        return double(s >> 11) * (1.0 / 9007199254740992.0);
    };
    P.assign(kNParams, 0.f);
    auto fill = [&](int off, int n_out, int n_in) {
        const double a = std::sqrt(6.0 / double(n_in + n_out));
        for (int k = 0; k < n_out * n_in; ++k) P[off + k] = float((2.0 * unif() - 1.0) * a);
    };
    fill(bhr::surr::kW1, bhr::surr::kH, bhr::surr::kIn);
    fill(bhr::surr::kW2, bhr::surr::kH, bhr::surr::kH);
    fill(bhr::surr::kW3, bhr::surr::kH, bhr::surr::kH);
    fill(bhr::surr::kW4, bhr::surr::kOut, bhr::surr::kH);
}

constexpr uint32_t kMagic = 0x53524842u;  // "BHRS"
constexpr uint32_t kVersion = 1;

}  // namespace

extern "C" {

int bhr_surrogate_default_config(bhr_surrogate_config* c) {
    if (!c) return fail(BHR_ERR_INVALID_ARG, "bhr_surrogate_default_config: NULL");
    std::memset(c, 0, sizeof *c);
    c->rc_lo = 6.0f;
    c->rc_hi = 200.0f;
    c->b_max = 60.0f;
    c->band = 2e-3f;
    c->t_eps = 1e-3f;
    c->t_scale = 0.125f;
    c->y_scale = 0.02f;
    c->escape_r = 1000.0f;
    return BHR_OK;
}

int bhr_surrogate_create(bhr_surrogate** out, int device, const bhr_surrogate_config* cfg, uint64_t seed) {
    if (!out) return fail(BHR_ERR_INVALID_ARG, "bhr_surrogate_create: NULL");
    *out = nullptr;
    bhr_surrogate_config c;
    if (cfg) c = *cfg;
    else bhr_surrogate_default_config(&c);
    if (!(c.rc_lo > 2.0f && c.rc_hi > c.rc_lo && c.b_max > 5.2f && c.band > 0.0f && c.t_eps > 0.0f &&
          c.y_scale > 0.0f && c.escape_r > c.rc_hi))
        return fail(BHR_ERR_INVALID_ARG, "bhr_surrogate_create: inconsistent configuration");
    int ndev = 0;
    if (cudaGetDeviceCount(&ndev) != cudaSuccess || device < 0 || device >= ndev)
        return fail(BHR_ERR_CUDA, "bhr_surrogate_create: no such CUDA device");
    cudaDeviceProp prop{};
    cudaGetDeviceProperties(&prop, device);
    if (prop.major * 10 + prop.minor != 103)
        return fail(BHR_ERR_UNSUPPORTED, "bhr_surrogate_create: this library is built for sm_103a only");
    DevGuard dg(device);
    bhr_surrogate* s = new bhr_surrogate();
    s->device = device;
    s->sms = prop.multiProcessorCount;
    s->norm = bhr::surr::Norm{c.rc_lo, c.rc_hi, c.b_max, c.t_eps, c.t_scale, c.y_scale, c.band, 1.0f / c.escape_r};
    std::vector<float> P;
    init_params(P, seed);
    cudaError_t e = cudaMalloc(&s->params, sizeof(float) * kNParams);
    if (e == cudaSuccess) e = cudaMalloc(&s->grads, sizeof(float) * kNParams * bhr::surr::kGradCopies);
    if (e == cudaSuccess) e = cudaMalloc(&s->adam_m, sizeof(float) * kNParams);
    if (e == cudaSuccess) e = cudaMalloc(&s->adam_v, sizeof(float) * kNParams);
    if (e == cudaSuccess) e = cudaMalloc(&s->stats, sizeof(unsigned long long) * 4);
    if (e == cudaSuccess) e = cudaMalloc(&s->tab_status, 2 * sizeof(int));
    if (e == cudaSuccess) e = cudaMemset(s->tab_status, 0, 2 * sizeof(int));
    if (e == cudaSuccess) e = cudaMemcpy(s->params, P.data(), sizeof(float) * kNParams, cudaMemcpyHostToDevice);
    if (e == cudaSuccess) e = cudaMemset(s->adam_m, 0, sizeof(float) * kNParams);
    if (e == cudaSuccess) e = cudaMemset(s->adam_v, 0, sizeof(float) * kNParams);
    for (SurrLane& L : s->lane) {
        for (int k = 0; e == cudaSuccess && k < 3; ++k) e = cudaEventCreate(&L.ev[k]);
        for (int k = 0; e == cudaSuccess && k < 3; ++k) e = cudaStreamCreateWithFlags(&L.side[k], cudaStreamNonBlocking);
        for (cudaEvent_t* ev : {&L.start, &L.fork, &L.band_ready, &L.join[0], &L.join[1], &L.join[2]})
            if (e == cudaSuccess) e = cudaEventCreateWithFlags(ev, cudaEventDisableTiming);
    }
    if (e != cudaSuccess) {
        bhr_surrogate_destroy(s);
        return fail(BHR_ERR_OOM, std::string("bhr_surrogate_create: ") + cudaGetErrorString(e));
    }
    *out = s;
    return BHR_OK;
}

int bhr_surrogate_destroy(bhr_surrogate* s) {
    if (!s) return BHR_OK;
    DevGuard dg(s->device);
    for (void* p : {(void*)s->params, (void*)s->grads, (void*)s->adam_m, (void*)s->adam_v, (void*)s->X,
                    (void*)s->lab, (void*)s->stats, (void*)s->tab_status, (void*)s->loss, (void*)s->staging})
        if (p) cudaFree(p);
    for (SurrLane& L : s->lane) {
        for (void* p : {(void*)L.q, (void*)L.fb, (void*)L.mask, (void*)L.band, (void*)L.etab, (void*)L.ctab})
            if (p) cudaFree(p);
        for (cudaEvent_t e : {L.ev[0], L.ev[1], L.ev[2], L.start, L.fork, L.band_ready, L.join[0], L.join[1], L.join[2]})
            if (e) cudaEventDestroy(e);
        for (cudaStream_t st : L.side)
            if (st) cudaStreamDestroy(st);
    }
    for (cudaStream_t& st : s->hs)
        if (st) cudaStreamDestroy(st);
    delete s;
    return BHR_OK;
}

int bhr_surrogate_generate(bhr_surrogate* s, int64_t n_orbits, int samples_per_orbit, uint64_t seed,
                           void* stream, uint64_t* counts) {
    if (!s || n_orbits <= 0 || samples_per_orbit < 2 || samples_per_orbit > 8)
        return fail(BHR_ERR_INVALID_ARG, "bhr_surrogate_generate: bad arguments (2..8 samples per orbit)");
    DevGuard dg(s->device);
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    const int64_t n = n_orbits * samples_per_orbit;
    if (s->X) cudaFree(s->X);
    if (s->lab) cudaFree(s->lab);
    s->X = nullptr;
    s->lab = nullptr;
    s->n_samples = 0;
    cudaError_t e = cudaMalloc(&s->X, sizeof(bhr::surr::TrainSample) * size_t(n));
    if (e == cudaSuccess) e = cudaMalloc(&s->lab, size_t(n));
    if (e != cudaSuccess) return fail(BHR_ERR_OOM, std::string("bhr_surrogate_generate: ") + cudaGetErrorString(e));
    e = cudaMemsetAsync(s->stats, 0, sizeof(unsigned long long) * 4, st);
    if (e == cudaSuccess)
        e = bhr::surr::launch_orbit_data(seed, n_orbits, samples_per_orbit, s->norm, 0.004, s->X, s->lab, s->stats,
                                         s->sms * 16, st);
    if (e != cudaSuccess) return cfail(e, "bhr_surrogate_generate");
    s->n_samples = n;
    if (counts) {
        unsigned long long h[4];
        e = cudaMemcpyAsync(h, s->stats, sizeof h, cudaMemcpyDeviceToHost, st);
        if (e == cudaSuccess) e = cudaStreamSynchronize(st);
        if (e != cudaSuccess) return cfail(e, "bhr_surrogate_generate");
        for (int k = 0; k < 3; ++k) counts[k] = h[k];
    }
    return BHR_OK;
}

int bhr_surrogate_train(bhr_surrogate* s, int steps, int batch, float lr_max, float lr_min, float w_capture,
                        uint64_t seed, void* stream, float* loss_out) {
    if (!s || steps <= 0 || batch <= 0 || batch % 32 != 0 || !(lr_max > 0.0f) || lr_min < 0.0f)
        return fail(BHR_ERR_INVALID_ARG, "bhr_surrogate_train: bad arguments (batch must be a multiple of 32)");
    if (!s->X || s->n_samples == 0) return fail(BHR_ERR_NOT_READY, "bhr_surrogate_train: generate training data first");
    DevGuard dg(s->device);
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    if (steps > s->loss_cap) {
        if (s->loss) cudaFree(s->loss);
        s->loss = nullptr;
        s->loss_cap = 0;
        cudaError_t e = cudaMalloc(&s->loss, sizeof(float) * 3 * size_t(steps));
        if (e != cudaSuccess) return fail(BHR_ERR_OOM, "bhr_surrogate_train: loss buffer");
        s->loss_cap = steps;
    }
    cudaError_t e = cudaMemsetAsync(s->loss, 0, sizeof(float) * 3 * size_t(steps), st);
    const int grid = s->sms;
    for (int k = 0; e == cudaSuccess && k < steps; ++k) {
        const double frac = steps > 1 ? double(k) / double(steps - 1) : 1.0;
        const float lr = float(lr_min + 0.5 * (lr_max - lr_min) * (1.0 + std::cos(3.141592653589793 * frac)));
        // the gradient copies are zeroed here once; each Adam step zeroes them after reading
        if (k == 0) e = cudaMemsetAsync(s->grads, 0, sizeof(float) * kNParams * bhr::surr::kGradCopies, st);
        if (e == cudaSuccess)
            e = bhr::surr::launch_train_step(s->params, s->X, s->lab, s->n_samples, nullptr, batch,
                                             seed + 0x632BE59BD9B4E019ull * uint64_t(s->adam_step + 1), 1.0f,
                                             w_capture, s->grads, s->loss + 3 * k, grid, st);
        if (e == cudaSuccess)
            e = bhr::surr::launch_adam(s->params, s->grads, s->adam_m, s->adam_v, ++s->adam_step, lr, 0.9f, 0.999f,
                                       1e-8f, st);
    }
    if (e != cudaSuccess) return cfail(e, "bhr_surrogate_train");
    if (loss_out) {
        std::vector<float> h(3 * size_t(steps));
        e = cudaMemcpyAsync(h.data(), s->loss, sizeof(float) * h.size(), cudaMemcpyDeviceToHost, st);
        if (e == cudaSuccess) e = cudaStreamSynchronize(st);
        if (e != cudaSuccess) return cfail(e, "bhr_surrogate_train");
        for (int k = 0; k < steps; ++k) {
            const float ny = h[3 * k + 2] > 0 ? h[3 * k + 2] : 1.0f;
            loss_out[2 * k] = h[3 * k] / ny;                 // mean squared error of y
            loss_out[2 * k + 1] = h[3 * k + 1] / float(batch);  // mean capture BCE
        }
    }
    return BHR_OK;
}

int bhr_surrogate_samples(bhr_surrogate* s, int64_t offset, int64_t n, float* out, int8_t* labels) {
    if (!s || !out || !labels || offset < 0 || n <= 0 || offset + n > s->n_samples)
        return fail(BHR_ERR_INVALID_ARG, "bhr_surrogate_samples: range outside the generated samples");
    DevGuard dg(s->device);
    cudaError_t e = cudaMemcpy(out, s->X + offset, sizeof(bhr::surr::TrainSample) * size_t(n), cudaMemcpyDeviceToHost);
    if (e == cudaSuccess) e = cudaMemcpy(labels, s->lab + offset, size_t(n), cudaMemcpyDeviceToHost);
    return e == cudaSuccess ? BHR_OK : cfail(e, "bhr_surrogate_samples");
}

int bhr_surrogate_params(bhr_surrogate* s, float* out, int n) {
    if (!s || !out || n != kNParams) return fail(BHR_ERR_INVALID_ARG, "bhr_surrogate_params: n must be the parameter count");
    DevGuard dg(s->device);
    cudaError_t e = cudaMemcpy(out, s->params, sizeof(float) * kNParams, cudaMemcpyDeviceToHost);
    return e == cudaSuccess ? BHR_OK : cfail(e, "bhr_surrogate_params");
}

int bhr_surrogate_set_params(bhr_surrogate* s, const float* in, int n) {
    if (!s || !in || n != kNParams) return fail(BHR_ERR_INVALID_ARG, "bhr_surrogate_set_params: n must be the parameter count");
    DevGuard dg(s->device);
    cudaError_t e = cudaMemcpy(s->params, in, sizeof(float) * kNParams, cudaMemcpyHostToDevice);
    return e == cudaSuccess ? BHR_OK : cfail(e, "bhr_surrogate_set_params");
}

int bhr_surrogate_param_count(void) { return kNParams; }

int bhr_surrogate_gradients(bhr_surrogate* s, const float* samples, const int8_t* labels, int n, float w_capture,
                            float* grad_out, float* loss_out) {
    if (!s || !samples || !labels || !grad_out || n <= 0 || n % 32 != 0)
        return fail(BHR_ERR_INVALID_ARG, "bhr_surrogate_gradients: n must be a positive multiple of 32");
    DevGuard dg(s->device);
    bhr::surr::TrainSample* X = nullptr;
    int8_t* L = nullptr;
    int64_t* idx = nullptr;
    float *G = nullptr, *loss = nullptr;
    std::vector<int64_t> hidx(static_cast<size_t>(n));
    for (int k = 0; k < n; ++k) hidx[size_t(k)] = k;
    cudaError_t e = cudaMalloc(&X, sizeof(bhr::surr::TrainSample) * size_t(n));
    if (e == cudaSuccess) e = cudaMalloc(&L, size_t(n));
    if (e == cudaSuccess) e = cudaMalloc(&idx, sizeof(int64_t) * size_t(n));
    if (e == cudaSuccess) e = cudaMalloc(&G, sizeof(float) * kNParams * bhr::surr::kGradCopies);
    if (e == cudaSuccess) e = cudaMalloc(&loss, sizeof(float) * 3);
    if (e == cudaSuccess) e = cudaMemcpy(X, samples, sizeof(bhr::surr::TrainSample) * size_t(n), cudaMemcpyHostToDevice);
    if (e == cudaSuccess) e = cudaMemcpy(L, labels, size_t(n), cudaMemcpyHostToDevice);
    if (e == cudaSuccess) e = cudaMemcpy(idx, hidx.data(), sizeof(int64_t) * size_t(n), cudaMemcpyHostToDevice);
    if (e == cudaSuccess) e = cudaMemset(G, 0, sizeof(float) * kNParams * bhr::surr::kGradCopies);
    if (e == cudaSuccess) e = cudaMemset(loss, 0, sizeof(float) * 3);
    if (e == cudaSuccess)
        e = bhr::surr::launch_train_step(s->params, X, L, n, idx, n, 0, 1.0f, w_capture, G, loss, s->sms, nullptr);
    std::vector<float> hg(size_t(kNParams) * bhr::surr::kGradCopies);
    if (e == cudaSuccess) e = cudaMemcpy(hg.data(), G, sizeof(float) * hg.size(), cudaMemcpyDeviceToHost);
    if (e == cudaSuccess)
        for (int k = 0; k < kNParams; ++k) {
            float acc = 0.f;
            for (int r = 0; r < bhr::surr::kGradCopies; ++r) acc += hg[size_t(r) * kNParams + k];
            grad_out[k] = acc;
        }
    float hl[3] = {0, 0, 0};
    if (e == cudaSuccess) e = cudaMemcpy(hl, loss, sizeof hl, cudaMemcpyDeviceToHost);
    for (void* p : {(void*)X, (void*)L, (void*)idx, (void*)G, (void*)loss})
        if (p) cudaFree(p);
    if (e != cudaSuccess) return cfail(e, "bhr_surrogate_gradients");
    if (loss_out) {
        loss_out[0] = hl[0];
        loss_out[1] = hl[1];
        loss_out[2] = hl[2];
    }
    return BHR_OK;
}

int bhr_surrogate_eval(bhr_surrogate* s, const float* queries, int n, float* out) {
    if (!s || !queries || !out || n <= 0) return fail(BHR_ERR_INVALID_ARG, "bhr_surrogate_eval: bad arguments");
    DevGuard dg(s->device);
    float4* q = nullptr;
    float2* o = nullptr;
    int* status = nullptr;
    int hstatus = 0;
    std::vector<float4> hq(static_cast<size_t>(n));
    for (int k = 0; k < n; ++k) hq[size_t(k)] = make_float4(queries[3 * k], queries[3 * k + 1], queries[3 * k + 2], 0.f);
    cudaError_t e = cudaMalloc(&q, sizeof(float4) * size_t(n));
    if (e == cudaSuccess) e = cudaMalloc(&o, sizeof(float2) * size_t(n));
    if (e == cudaSuccess) e = cudaMalloc(&status, sizeof(int));
    if (e == cudaSuccess) e = cudaMemset(status, 0, sizeof(int));
    if (e == cudaSuccess) e = cudaMemcpy(q, hq.data(), sizeof(float4) * size_t(n), cudaMemcpyHostToDevice);
    if (e == cudaSuccess) e = bhr::surr::launch_mlp_infer(s->params, q, o, n, status, s->sms * 3, nullptr);
    if (e == cudaSuccess) e = cudaMemcpy(out, o, sizeof(float2) * size_t(n), cudaMemcpyDeviceToHost);
    if (e == cudaSuccess) e = cudaMemcpy(&hstatus, status, sizeof(int), cudaMemcpyDeviceToHost);
    if (q) cudaFree(q);
    if (o) cudaFree(o);
    if (status) cudaFree(status);
    if (e != cudaSuccess) return cfail(e, "bhr_surrogate_eval");
    return hstatus ? fail(BHR_ERR_TIMEOUT, "bhr_surrogate_eval: a tensor-core completion wait ran out") : BHR_OK;
}

int bhr_surrogate_wait_selftest(bhr_surrogate* s) {
    if (!s) return fail(BHR_ERR_INVALID_ARG, "bhr_surrogate_wait_selftest: NULL");
    DevGuard dg(s->device);
    constexpr int n = 128;  // one tile, one block
    float4* q = nullptr;
    float2* o = nullptr;
    int* status = nullptr;
    int hstatus = 0;
    cudaError_t e = cudaMalloc(&q, sizeof(float4) * n);
    if (e == cudaSuccess) e = cudaMalloc(&o, sizeof(float2) * n);
    if (e == cudaSuccess) e = cudaMalloc(&status, sizeof(int));
    if (e == cudaSuccess) e = cudaMemset(q, 0, sizeof(float4) * n);
    if (e == cudaSuccess) e = cudaMemset(status, 0, sizeof(int));
    if (e == cudaSuccess) e = bhr::surr::launch_mlp_infer(s->params, q, o, n, status, 1, nullptr, 100000000ll, true);
    if (e == cudaSuccess) e = cudaMemcpy(&hstatus, status, sizeof(int), cudaMemcpyDeviceToHost);
    if (q) cudaFree(q);
    if (o) cudaFree(o);
    if (status) cudaFree(status);
    if (e != cudaSuccess) return cfail(e, "bhr_surrogate_wait_selftest");
    return hstatus ? fail(BHR_ERR_TIMEOUT, "bhr_surrogate_wait_selftest: the withheld completions timed out and were reported")
                   : fail(BHR_ERR_CUDA, "bhr_surrogate_wait_selftest: the withheld completions were not reported");
}

int bhr_surrogate_save(bhr_surrogate* s, const char* path) {
    if (!s || !path) return fail(BHR_ERR_INVALID_ARG, "bhr_surrogate_save: NULL");
    std::vector<float> P(kNParams);
    const int rc = bhr_surrogate_params(s, P.data(), kNParams);
    if (rc != BHR_OK) return rc;
    FILE* f = std::fopen(path, "wb");
    if (!f) return fail(BHR_ERR_IO, std::string("bhr_surrogate_save: cannot open ") + path);
    const uint32_t hdr[3] = {kMagic, kVersion, uint32_t(kNParams)};
    bool ok = std::fwrite(hdr, sizeof hdr, 1, f) == 1 && std::fwrite(&s->norm, sizeof s->norm, 1, f) == 1 &&
              std::fwrite(&s->adam_step, sizeof s->adam_step, 1, f) == 1 &&
              std::fwrite(P.data(), sizeof(float), P.size(), f) == P.size();
    ok = (std::fclose(f) == 0) && ok;
    return ok ? BHR_OK : fail(BHR_ERR_IO, "bhr_surrogate_save: write failed");
}

int bhr_surrogate_load(bhr_surrogate* s, const char* path) {
    if (!s || !path) return fail(BHR_ERR_INVALID_ARG, "bhr_surrogate_load: NULL");
    FILE* f = std::fopen(path, "rb");
    if (!f) return fail(BHR_ERR_IO, std::string("bhr_surrogate_load: cannot open ") + path);
    uint32_t hdr[3];
    bhr::surr::Norm nm{};
    int step = 0;
    std::vector<float> P(kNParams);
    bool ok = std::fread(hdr, sizeof hdr, 1, f) == 1 && hdr[0] == kMagic && hdr[1] == kVersion &&
              hdr[2] == uint32_t(kNParams) && std::fread(&nm, sizeof nm, 1, f) == 1 &&
              std::fread(&step, sizeof step, 1, f) == 1 && std::fread(P.data(), sizeof(float), P.size(), f) == P.size();
    std::fclose(f);
    if (!ok) return fail(BHR_ERR_IO, std::string("bhr_surrogate_load: not a surrogate file: ") + path);
    s->norm = nm;
    s->adam_step = step;
    return bhr_surrogate_set_params(s, P.data(), kNParams);
}

namespace {
int surrogate_trace_lane(bhr_surrogate* s, const bhr_view* views, int nviews, bhr_hit* const* out_dev, void* stream,
                         int lane);
}

}  // extern "C"

namespace bhr {
namespace surr {
bool supports_view(const Norm& nm, const bhr_view& v, std::string* why) {
    if (!v.lensing || v.far_mode) {
        *why = "the surrogate answers lensed rays (lensing on, not far mode)";
        return false;
    }
    if (v.disk_mode != BHR_DISK_NONE && v.disk_mode != BHR_DISK_THIN) {
        *why = "the surrogate answers the thin disk or none";
        return false;
    }
    if (v.term_mode == BHR_TERM_CONFIG) {
        if (std::fabs(1.0f / v.escape_r - nm.ue) > 1e-9f) {
            *why = "the CONFIG rule's escape radius differs from the trained exit radius";
            return false;
        }
        return true;
    }
    // SHADER and CPU: the tolerance escape; exit_u_tol converges to float precision for
    // tolerances up to the shader's ESC_TOL (0.01)
    const float rmin = v.term_mode == BHR_TERM_SHADER ? bhr::host::shader_r_esc_min(v.disk_outer) : v.r_esc_min;
    if (!(v.esc_tol > 0.0f && v.esc_tol <= 0.01f) || !(rmin > 3.0f) || !(1.0f / rmin > nm.ue)) {
        *why = "the tolerance escape needs 0 < esc_tol <= 0.01 and 3 < rEscMin < the trained exit radius";
        return false;
    }
    return true;
}
Norm norm_of(const bhr_surrogate* s) { return s->norm; }
int device_of(const bhr_surrogate* s) { return s->device; }
}  // namespace surr
}  // namespace bhr

extern "C" {

int bhr_surrogate_trace(bhr_surrogate* s, const bhr_view* views, int nviews, bhr_hit* const* out_dev, void* stream) {
    return surrogate_trace_lane(s, views, nviews, out_dev, stream, 0);
}

namespace {
// bhr_surrogate_trace on the side streams of pipeline lane `lane`.
int surrogate_trace_lane(bhr_surrogate* s, const bhr_view* views, int nviews, bhr_hit* const* out_dev, void* stream,
                         int lane) {
    if (!s || !views || nviews <= 0 || !out_dev) return fail(BHR_ERR_INVALID_ARG, "bhr_surrogate_trace: bad arguments");
    int64_t biggest = 0;
    for (int k = 0; k < nviews; ++k) {
        std::string msg;
        const int rc = bhr::host::check_view(views[k], k, &msg);
        if (rc != BHR_OK) return fail(rc, "bhr_surrogate_trace: " + msg);
        std::string why;
        if (!bhr::surr::supports_view(s->norm, views[k], &why))
            return fail(BHR_ERR_UNSUPPORTED, "bhr_surrogate_trace: view " + std::to_string(k) + ": " + why);
        if (!out_dev[k] || reinterpret_cast<uintptr_t>(out_dev[k]) % 16 != 0)
            return fail(BHR_ERR_INVALID_ARG, "bhr_surrogate_trace: output buffers must be 16-byte aligned");
        biggest = std::max<int64_t>(biggest, int64_t(views[k].width) * views[k].height);
    }
    DevGuard dg(s->device);
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    // per-view fallback lists, one after the other
    std::vector<int64_t> off(size_t(nviews) + 1, 0);
    for (int k = 0; k < nviews; ++k) off[size_t(k) + 1] = off[size_t(k)] + int64_t(views[k].width) * views[k].height;
    SurrLane& L = s->lane[lane];
    // what plans point into: lane 0's work memory (plans run on lane 0)
    auto plan_memory = [&] {
        return std::array<uintptr_t, 12>{uintptr_t(L.fb),   uintptr_t(L.fb_cap),   uintptr_t(L.q),
                                         uintptr_t(L.nq),   uintptr_t(L.etab),     uintptr_t(L.etab_cap),
                                         uintptr_t(L.ctab), uintptr_t(L.ctab_cap), uintptr_t(L.mask),
                                         uintptr_t(L.mask_cap), uintptr_t(L.band), uintptr_t(L.band_cap)};
    };
    const auto before = plan_memory();
    // per-view band masks, one after the other (ceil(rays / 32) words each)
    std::vector<int64_t> moff(size_t(nviews) + 1, 0);
    for (int k = 0; k < nviews; ++k) moff[size_t(k) + 1] = moff[size_t(k)] + (int64_t(views[k].width) * views[k].height + 31) / 32;
    const int64_t nq = 4 * int64_t(nviews) + 2;
    cudaError_t e = grow(&L.fb, &L.fb_cap, off[size_t(nviews)]);
    if (e == cudaSuccess) e = grow(&L.q, &L.nq, nq);
    if (e == cudaSuccess) e = grow(&L.mask, &L.mask_cap, moff[size_t(nviews)]);
    if (e == cudaSuccess) e = grow(&L.band, &L.band_cap, int64_t(bhr::surr::kBandCap) * nviews);
    constexpr int64_t kTab = bhr::surr::kExitTabEntries;  // table entries per view
    if (e == cudaSuccess) e = grow(&L.etab, &L.etab_cap, kTab * std::max<int64_t>(nviews, 64));
    constexpr int64_t kCells = bhr::surr::kCrossCells;
    if (e == cudaSuccess) e = grow(&L.ctab, &L.ctab_cap, kCells * std::max<int64_t>(nviews, 16));
    if (lane == 0 && plan_memory() != before) ++s->work_gen;
    if (e != cudaSuccess) return fail(BHR_ERR_OOM, "bhr_surrogate_trace: work memory");
    bhr::WorkQueue* const qb = L.q + 2 * nviews + 1;  // the band march's queues
    // the views' constants
    std::vector<bhr::surr::SurrView> svs(static_cast<size_t>(nviews));
    std::vector<bhr::DevView> dvs(static_cast<size_t>(nviews));
    std::vector<bhr::Rule> rules(static_cast<size_t>(nviews));
    bool one_rule = true;
    for (int k = 0; k < nviews; ++k) {
        bhr::surr::SurrView& sv = svs[size_t(k)];
        sv.view = bhr::host::make_dev_view(views[k], out_dev[k]);
        sv.view.list_off = off[size_t(k)];
        sv.rule = bhr::host::make_rule(views[k]);
        sv.norm = s->norm;
        sv.x1 = float((std::log(double(sv.view.rcam)) - std::log(double(s->norm.rc_lo))) /
                          (std::log(double(s->norm.rc_hi)) - std::log(double(s->norm.rc_lo))) * 2.0 - 1.0);
        sv.uc = 1.0f / sv.view.rcam;
        sv.u_esc_min = sv.rule.r_esc_min > 0.0f ? 1.0f / sv.rule.r_esc_min : 1.0f;
        sv.b_kink = views[k].term_mode == BHR_TERM_CONFIG ? 0.0f : tolerance_kink(sv.rule.esc_tol, sv.u_esc_min);
        sv.exit_table = L.etab + kTab * k;
        bhr::surr::exit_table_range(s->norm, sv.tab_lo, sv.tab_h);
        for (int h = 0; h < 2; ++h) sv.tab_inv_h[h] = 1.0f / sv.tab_h[h];
        sv.cross_table = L.ctab + kCells * k;
        sv.cx_h = sv.tab_h[1] * float(bhr::surr::kExitTableN - 1) / float(bhr::surr::kCrossNx - 1);
        sv.cx_inv_h = 1.0f / sv.cx_h;
        {
            const double cx = views[k].cam_pos[0], cy = views[k].cam_pos[1], cz = views[k].cam_pos[2];
            const double rc = std::sqrt(cx * cx + cy * cy + cz * cz);
            bhr::surr::Fp64Cam& fc = sv.fc;
            fc.inv_w2 = 2.0 / double(views[k].width);
            fc.inv_h2 = 2.0 / double(views[k].height);
            fc.aspect_d = double(views[k].width) / double(views[k].height);
            fc.rhat_d[0] = cx / rc;
            fc.rhat_d[1] = cy / rc;
            fc.rhat_d[2] = cz / rc;
            fc.b_scale_d = rc / std::sqrt(std::max(1.0 - 2.0 / rc, 1e-300));
            sv.b_scale = float(fc.b_scale_d);
            // the pixel direction before normalisation, B (cx, cy, -1) with cx, cy affine in the
            // pixel (blackhole.frag:68-72), about the image's centre
            const bhr::DevView& dv = sv.view;
            const double th = double(dv.tan_half), asp = double(dv.aspect);
            sv.i_mid = views[k].width / 2;
            sv.j_mid = views[k].height / 2;
            const double sx = fc.inv_w2 * th * asp, sy = fc.inv_h2 * th;
            const double cx0 = ((double(sv.i_mid) + 0.5 + double(dv.jitter[0])) * fc.inv_w2 - 1.0) * th * asp;
            const double cy0 = ((double(sv.j_mid) + 0.5 + double(dv.jitter[1])) * fc.inv_h2 - 1.0) * th;
            for (int c = 0; c < 3; ++c) {
                sv.dir_i[c] = float(double(dv.basis[c]) * sx);
                sv.dir_j[c] = float(double(dv.basis[3 + c]) * sy);
                sv.dir_0[c] = float(double(dv.basis[c]) * cx0 + double(dv.basis[3 + c]) * cy0 - double(dv.basis[6 + c]));
            }
            // the camera's tangential ray has b = b_scale_d
            const double beta_t = fc.b_scale_d / 5.196152422706632 - 1.0;
            const double x2_t = std::log1p(beta_t / double(s->norm.t_eps)) * double(s->norm.t_scale);
            sv.x2_lim = float(x2_t - double(bhr::surr::kTangentMargin) * double(sv.tab_h[1]));
        }
        sv.band_mask = nullptr;
        dvs[size_t(k)] = sv.view;
        rules[size_t(k)] = sv.rule;
        one_rule = one_rule && std::memcmp(&rules[0], &sv.rule, sizeof sv.rule) == 0;
    }
    // the band march: the views' band rays found before the pass and marched beside it (views that
    // share one rule, as the fallback march's multi-view launch needs; views whose rows the search
    // cannot bound keep their band rays on the fallback list)
    const bool band = one_rule && nviews <= bhr::kMaxViews;
    static thread_local bhr::surr::BandBatch bb;
    if (band) {
        bb.nviews = nviews;
        bb.rule = rules[0];
        bb.band = s->norm.band;
        bb.qb = qb;
        int rows = 0;
        const double s27 = 5.196152422706632, margin = 2.0 * double(s->norm.band);
        for (int k = 0; k < nviews; ++k) {
            bhr::surr::BandView& bv = bb.v[k];
            bhr::surr::SurrView& sv = svs[size_t(k)];
            bv.view = sv.view;
            bv.fc = sv.fc;
            bv.mask = L.mask + moff[size_t(k)];
            bv.list = L.band + int64_t(bhr::surr::kBandCap) * k;
            bv.row0 = rows;
            bv.rows = bhr::surr::band_rows(views[k], sv.fc, s27 - margin, s27 + margin, &bv.q) ? views[k].height : 0;
            rows += bv.rows;
            sv.band_mask = bv.mask;
            dvs[size_t(k)].list_off = int64_t(bhr::surr::kBandCap) * k;
        }
        bb.total_rows = rows;
    }
    e = cudaMemsetAsync(L.q, 0, sizeof(bhr::WorkQueue) * size_t(nq), st);
    if (e == cudaSuccess) e = cudaMemsetAsync(s->tab_status + lane, 0, sizeof(int), st);
    if (e == cudaSuccess && band) e = cudaMemsetAsync(L.mask, 0, sizeof(uint32_t) * size_t(moff[size_t(nviews)]), st);
    if (e == cudaSuccess) e = cudaEventRecord(L.ev[0], st);
    // 1) on side[2]: the band rays of every view (lists and masks), then their march, which runs
    // beside the tables and the passes (64-thread blocks: they leave the SMs' registers to the pass)
    if (e == cudaSuccess && band) {
        e = cudaEventRecord(L.start, st);
        if (e == cudaSuccess) e = cudaStreamWaitEvent(L.side[2], L.start, 0);
        if (e == cudaSuccess) e = bhr::surr::launch_band_list(bb, L.side[2]);
        if (e == cudaSuccess) e = cudaEventRecord(L.band_ready, L.side[2]);
        static thread_local bhr::ViewBatch vb;
        vb.nviews = nviews;
        vb.rule = rules[0];
        vb.total_chunks = 0;
        for (int k = 0; k < nviews; ++k) vb.views[k] = dvs[size_t(k)];
        bhr::LaunchCfg cfg{};
        cfg.block = 64;
        cfg.chunk = 32;
        cfg.refill = 8;
        cfg.variant = bhr::rule_variant(vb.rule);
        cfg.grid = s->sms;
        const bhr::Scratch sc{qb + 2 * nviews, nullptr, nullptr};
        if (e == cudaSuccess) e = bhr::launch_march_multi_list(vb, sc, L.band, qb, cfg, L.side[2]);
        if (e == cudaSuccess) e = cudaEventRecord(L.join[2], L.side[2]);
        for (int k = 0; k < nviews; ++k) dvs[size_t(k)].list_off = off[size_t(k)];
    }
    // 2) the learned surrogate's tables of every view: one launch on the tensor cores per 64 views
    const bool net = s->use_network;
    uint64_t net_rows = 0;
    if (net) {
        static thread_local bhr::surr::TabBatch tb;
        for (int k0 = 0; e == cudaSuccess && k0 < nviews; k0 += bhr::surr::kTabMaxViews) {
            const int k1 = std::min(nviews, k0 + bhr::surr::kTabMaxViews);
            tb.nviews = k1 - k0;
            tb.norm = s->norm;
            for (int h = 0; h < 2; ++h) {
                tb.tab_lo[h] = svs[0].tab_lo[h];
                tb.tab_h[h] = svs[0].tab_h[h];
            }
            tb.cx_h = svs[0].cx_h;
            int tiles = 0;
            for (int k = k0; k < k1; ++k) {
                const bhr::surr::SurrView& sv = svs[size_t(k)];
                bhr::surr::TabView& tv = tb.v[k - k0];
                tv.x1 = sv.x1;
                tv.uc = sv.uc;
                tv.u_esc_min = sv.u_esc_min;
                tv.esc_tol = sv.rule.esc_tol;
                tv.b_kink = sv.b_kink;
                tv.two_over_r3 = sv.view.two_over_r3;
                tv.disk_inner = sv.rule.disk_inner;
                tv.disk_outer = sv.rule.disk_outer;
                tv.tol = views[k].term_mode != BHR_TERM_CONFIG;
                tv.tile0 = tiles;
                tv.exit_table = L.etab + kTab * k;
                tv.cross_table = L.ctab + kCells * k;
                tiles += bhr::surr::tab_tiles(tv.tol != 0);
            }
            tb.ntiles = tiles;
            net_rows += uint64_t(tiles) * 128u;
            e = bhr::surr::launch_tables(tb, s->params, s->tab_status + lane, s->sms * 4, st);
        }
    }
    if (e == cudaSuccess) e = cudaEventRecord(L.fork, st);
    for (int j = 0; e == cudaSuccess && j < 2; ++j) {
        e = cudaStreamWaitEvent(L.side[j], L.fork, 0);
        if (e == cudaSuccess && band) e = cudaStreamWaitEvent(L.side[j], L.band_ready, 0);
    }
    // 3) the surrogate pass of every view (the non-learned variant builds its exit table first),
    // alternating between side[0] and side[1]
    for (int k = 0; e == cudaSuccess && k < nviews; ++k) {
        const bhr::surr::SurrView& sv = svs[size_t(k)];
        cudaStream_t vs = L.side[k & 1];
        if (!net) e = bhr::surr::launch_exit_table_cf(sv, L.etab + kTab * k, vs);
        if (e == cudaSuccess)
            e = bhr::surr::launch_surrogate_trace(sv, L.q + 2 * k, L.fb + off[size_t(k)],
                                                  s->sms * bhr::surr::surr_blocks_per_sm(net), net, vs);
    }
    for (int j = 0; e == cudaSuccess && j < 2; ++j) {
        e = cudaEventRecord(L.join[j], L.side[j]);
        if (e == cudaSuccess) e = cudaStreamWaitEvent(st, L.join[j], 0);
    }
    if (e == cudaSuccess) e = cudaEventRecord(L.ev[1], st);
    // 4) the integrator on the rays the pass sent to the fallback list: one launch for all views
    // when they share a rule. The rays are few and the near-critical ones long: claims of 32
    // spread them over as many warps as possible, so the launch ends with its slowest ray
    bhr::LaunchCfg cfg{};
    cfg.block = 512;
    cfg.chunk = 32;
    cfg.refill = 8;
    if (e == cudaSuccess && one_rule && nviews <= bhr::kMaxViews) {
        static thread_local bhr::ViewBatch b;
        b.nviews = nviews;
        b.rule = rules[0];
        b.total_chunks = 0;
        for (int k = 0; k < nviews; ++k) b.views[k] = dvs[size_t(k)];
        cfg.variant = bhr::rule_variant(b.rule);
        // one block per SM: the list is usually empty (the band march took the band rays), and
        // 16 warps per SM still spread a few thousand rays in claims of 32
        cfg.grid = s->sms;
        const bhr::Scratch sc{L.q + 2 * nviews, nullptr, nullptr};
        e = bhr::launch_march_multi_list(b, sc, L.fb, L.q, cfg, st);
    } else {
        for (int k = 0; e == cudaSuccess && k < nviews; ++k) {
            cfg.variant = bhr::rule_variant(rules[size_t(k)]);
            cfg.grid = s->sms * std::max(1, bhr::march_blocks_per_sm(512, cfg.variant, false, false));
            const bhr::Scratch sc{L.q + 2 * k + 1, nullptr, nullptr};
            e = bhr::launch_march_list(dvs[size_t(k)], rules[size_t(k)], sc, L.fb + off[size_t(k)],
                                       &L.q[2 * k].fb_count, cfg, st);
        }
    }
    // the trace ends with the band march too
    if (e == cudaSuccess && band) e = cudaStreamWaitEvent(st, L.join[2], 0);
    if (e == cudaSuccess) e = cudaEventRecord(L.ev[2], st);
    if (e != cudaSuccess) return cfail(e, "bhr_surrogate_trace");
    // a trace recorded into a graph (plan creation and update) runs nothing now: its event
    // records are capture dependencies, not timings, so the last executed trace stays the one
    // bhr_surrogate_trace_times and bhr_surrogate_trace_stats report
    cudaStreamCaptureStatus cs = cudaStreamCaptureStatusNone;
    e = cudaStreamIsCapturing(st, &cs);
    if (e != cudaSuccess) return cfail(e, "bhr_surrogate_trace: capture status");
    if (cs == cudaStreamCaptureStatusNone) {
        s->last_stream = st;
        s->last_lane = lane;
        s->last_nviews = nviews;
        s->last_rows = net_rows;
        s->have_last = true;
        s->last_from_plan = false;
    }
    return BHR_OK;
}
}  // namespace

// A fixed batch of views traced by one CUDA graph of bhr_surrogate_trace (bhr_surrogate_plan_*).
struct bhr_surrogate_plan {
    bhr_surrogate* s = nullptr;
    cudaStream_t cap = nullptr;
    cudaGraph_t graph = nullptr;
    cudaGraphExec_t exec = nullptr;
    int nviews = 0;
    uint64_t work_gen = 0;  // the surrogate's work memory generation the graph was captured with
    uint64_t rows = 0;      // network rows of a replay (the views' tables)
    std::vector<bhr_view> views;  // the views and outputs of the captured trace
    std::vector<bhr_hit*> outs;
};

int bhr_surrogate_plan_destroy(bhr_surrogate_plan* p) {
    if (!p) return BHR_OK;
    DevGuard dg(p->s->device);
    if (p->s->have_last && p->s->last_stream) cudaStreamSynchronize(p->s->last_stream);
    if (p->exec) cudaGraphExecDestroy(p->exec);
    if (p->graph) cudaGraphDestroy(p->graph);
    if (p->cap) {
        cudaStreamSynchronize(p->cap);
        cudaStreamDestroy(p->cap);
    }
    delete p;
    return BHR_OK;
}

int bhr_surrogate_plan_create(bhr_surrogate* s, const bhr_view* views, int nviews, bhr_hit* const* out_dev,
                              bhr_surrogate_plan** out) {
    if (!s || !out) return fail(BHR_ERR_INVALID_ARG, "bhr_surrogate_plan_create: NULL argument");
    *out = nullptr;
    bhr_surrogate_plan* p = new (std::nothrow) bhr_surrogate_plan();
    if (!p) return fail(BHR_ERR_OOM, "bhr_surrogate_plan_create: out of host memory");
    p->s = s;
    p->nviews = nviews;
    DevGuard dg(s->device);
    cudaError_t e = cudaStreamCreateWithFlags(&p->cap, cudaStreamNonBlocking);
    if (e != cudaSuccess) {
        bhr_surrogate_plan_destroy(p);
        return cfail(e, "bhr_surrogate_plan_create: stream");
    }
    // one eager trace: checks the views, sizes the work memory, sets the kernel attributes
    int rc = bhr_surrogate_trace(s, views, nviews, out_dev, p->cap);
    if (rc == BHR_OK) {
        e = cudaStreamSynchronize(p->cap);
        if (e != cudaSuccess) rc = cfail(e, "bhr_surrogate_plan_create: first trace");
        p->rows = s->last_rows;
    }
    if (rc == BHR_OK) {
        e = cudaStreamBeginCapture(p->cap, cudaStreamCaptureModeThreadLocal);
        if (e != cudaSuccess) rc = cfail(e, "bhr_surrogate_plan_create: begin capture");
    }
    if (rc == BHR_OK) {
        const int rt = bhr_surrogate_trace(s, views, nviews, out_dev, p->cap);
        e = cudaStreamEndCapture(p->cap, &p->graph);
        if (rt != BHR_OK) rc = rt;
        else if (e != cudaSuccess) rc = cfail(e, "bhr_surrogate_plan_create: end capture");
    }
    if (rc == BHR_OK) {
        e = cudaGraphInstantiate(&p->exec, p->graph, 0);
        if (e != cudaSuccess) rc = cfail(e, "bhr_surrogate_plan_create: instantiate");
    }
    p->work_gen = s->work_gen;
    if (rc == BHR_OK) {
        p->views.assign(views, views + nviews);
        p->outs.assign(out_dev, out_dev + nviews);
    }
    if (rc != BHR_OK) {
        bhr_surrogate_plan_destroy(p);
        return rc;
    }
    *out = p;
    return BHR_OK;
}

int bhr_surrogate_plan_update(bhr_surrogate_plan* p, const bhr_view* views, int nviews) {
    if (!p || !p->exec) return fail(BHR_ERR_INVALID_ARG, "bhr_surrogate_plan_update: plan is NULL or empty");
    if (!views || nviews != p->nviews) return fail(BHR_ERR_INVALID_ARG, "bhr_surrogate_plan_update: the view count must stay the same");
    for (int k = 0; k < nviews; ++k)
        if (views[k].width != p->views[size_t(k)].width || views[k].height != p->views[size_t(k)].height)
            return fail(BHR_ERR_INVALID_ARG, "bhr_surrogate_plan_update: view " + std::to_string(k) +
                                                 " changes its size; create a new plan");
    bhr_surrogate* s = p->s;
    if (p->work_gen != s->work_gen)
        return fail(BHR_ERR_NOT_READY, "bhr_surrogate_plan_update: the surrogate's work memory was reallocated; "
                                       "recreate the plan");
    DevGuard dg(s->device);
    cudaGraph_t g = nullptr;
    cudaError_t e = cudaStreamBeginCapture(p->cap, cudaStreamCaptureModeThreadLocal);
    if (e != cudaSuccess) return cfail(e, "bhr_surrogate_plan_update: begin capture");
    int rc = surrogate_trace_lane(s, views, nviews, p->outs.data(), p->cap, 0);
    e = cudaStreamEndCapture(p->cap, &g);
    if (rc == BHR_OK && e != cudaSuccess) rc = cfail(e, "bhr_surrogate_plan_update: end capture");
    if (rc == BHR_OK && s->work_gen != p->work_gen)  // same sizes: nothing may have been reallocated
        rc = fail(BHR_ERR_NOT_READY, "bhr_surrogate_plan_update: the work memory changed during the update");
    if (rc == BHR_OK) {
        cudaGraphExecUpdateResultInfo info{};
        e = cudaGraphExecUpdate(p->exec, g, &info);
        if (e != cudaSuccess) {  // a changed topology: instantiate afresh
            cudaGetLastError();
            cudaGraphExec_t x = nullptr;
            e = cudaGraphInstantiate(&x, g, 0);
            if (e == cudaSuccess) {
                cudaGraphExecDestroy(p->exec);
                p->exec = x;
            } else {
                rc = cfail(e, "bhr_surrogate_plan_update: instantiate");
            }
        }
    }
    if (rc == BHR_OK) {
        if (p->graph) cudaGraphDestroy(p->graph);
        p->graph = g;
        p->views.assign(views, views + nviews);
    } else if (g) {
        cudaGraphDestroy(g);
    }
    return rc;
}

int bhr_surrogate_plan_launch(bhr_surrogate_plan* p, void* stream) {
    if (!p || !p->exec) return fail(BHR_ERR_INVALID_ARG, "bhr_surrogate_plan_launch: plan is NULL or empty");
    DevGuard dg(p->s->device);
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    if (p->work_gen != p->s->work_gen)
        return fail(BHR_ERR_NOT_READY,
                    "bhr_surrogate_plan_launch: a larger trace reallocated the surrogate's work memory since this plan "
                    "was made; destroy and recreate the plan");
    const cudaError_t e = cudaGraphLaunch(p->exec, st);
    if (e != cudaSuccess) return cfail(e, "bhr_surrogate_plan_launch");
    p->s->last_stream = st;
    p->s->last_lane = 0;
    p->s->last_nviews = p->nviews;
    p->s->last_rows = p->rows;
    p->s->have_last = true;
    p->s->last_from_plan = true;
    return BHR_OK;
}

int bhr_surrogate_trace_times(bhr_surrogate* s, float* ms2) {
    if (!s || !ms2) return fail(BHR_ERR_INVALID_ARG, "bhr_surrogate_trace_times: NULL");
    if (!s->have_last) return fail(BHR_ERR_NOT_READY, "bhr_surrogate_trace_times: no trace yet");
    if (s->last_from_plan)
        return fail(BHR_ERR_NOT_READY, "bhr_surrogate_trace_times: phase times come from bhr_surrogate_trace, not from plan replays");
    DevGuard dg(s->device);
    const SurrLane& L = s->lane[s->last_lane];
    cudaError_t e = cudaEventSynchronize(L.ev[2]);
    if (e == cudaSuccess) e = cudaEventElapsedTime(&ms2[0], L.ev[0], L.ev[1]);
    if (e == cudaSuccess) e = cudaEventElapsedTime(&ms2[1], L.ev[1], L.ev[2]);
    return e == cudaSuccess ? BHR_OK : cfail(e, "bhr_surrogate_trace_times");
}

int bhr_surrogate_trace_host(bhr_surrogate* s, const bhr_view* views, int nviews, bhr_hit* const* out_host) {
    if (!s || !views || nviews <= 0 || !out_host) return fail(BHR_ERR_INVALID_ARG, "bhr_surrogate_trace_host: bad arguments");
    int64_t biggest = 0;
    for (int k = 0; k < nviews; ++k) {
        if (!out_host[k]) return fail(BHR_ERR_INVALID_ARG, "bhr_surrogate_trace_host: output buffer is NULL");
        biggest = std::max<int64_t>(biggest, int64_t(views[k].width) * views[k].height);
    }
    DevGuard dg(s->device);
    const int64_t half = std::max<int64_t>(biggest, int64_t(1) << 22);
    cudaError_t e = cudaSuccess;
    if (half > s->staging_rays) {
        if (s->staging) cudaFree(s->staging);
        s->staging = nullptr;
        s->staging_rays = 0;
        e = cudaMalloc(&s->staging, sizeof(bhr_hit) * size_t(2 * half));
        if (e != cudaSuccess) return fail(BHR_ERR_OOM, "bhr_surrogate_trace_host: staging");
        s->staging_rays = half;
    }
    for (int k = 0; e == cudaSuccess && k < 2; ++k)
        if (!s->hs[k]) e = cudaStreamCreateWithFlags(&s->hs[k], cudaStreamNonBlocking);
    if (e != cudaSuccess) return cfail(e, "bhr_surrogate_trace_host");
    int rc = BHR_OK;
    std::vector<bhr_hit*> dst;
    int g = 0;
    // groups of views that fit one staging half; the group's records go to the host on its
    // stream while the next group is traced on the other
    for (int k0 = 0; rc == BHR_OK && k0 < nviews; ++g) {
        int k1 = k0;
        int64_t acc = 0;
        while (k1 < nviews && k1 - k0 < bhr::kMaxViews) {
            const int64_t n = int64_t(views[k1].width) * views[k1].height;
            if (acc + n > s->staging_rays && k1 > k0) break;
            acc += n;
            ++k1;
        }
        cudaStream_t st = s->hs[g & 1];
        bhr_hit* base = s->staging + (g & 1) * s->staging_rays;
        dst.clear();
        int64_t off = 0;
        for (int k = k0; k < k1; ++k) {
            dst.push_back(base + off);
            off += int64_t(views[k].width) * views[k].height;
        }
        rc = surrogate_trace_lane(s, views + k0, k1 - k0, dst.data(), st, g & 1);
        off = 0;
        for (int k = k0; rc == BHR_OK && k < k1; ++k) {
            const int64_t n = int64_t(views[k].width) * views[k].height;
            e = cudaMemcpyAsync(out_host[k], base + off, sizeof(bhr_hit) * size_t(n), cudaMemcpyDeviceToHost, st);
            if (e != cudaSuccess) rc = cfail(e, "bhr_surrogate_trace_host: copy");
            off += n;
        }
        k0 = k1;
    }
    for (cudaStream_t st : s->hs) {
        e = cudaStreamSynchronize(st);
        if (e != cudaSuccess && rc == BHR_OK) rc = cfail(e, "bhr_surrogate_trace_host: synchronize");
    }
    return rc;
}

int bhr_surrogate_use_network(bhr_surrogate* s, int use_network) {
    if (!s) return fail(BHR_ERR_INVALID_ARG, "bhr_surrogate_use_network: NULL");
    s->use_network = use_network != 0;
    return BHR_OK;
}

int bhr_surrogate_trace_stats(bhr_surrogate* s, uint64_t* out) {
    if (!s || !out) return fail(BHR_ERR_INVALID_ARG, "bhr_surrogate_trace_stats: NULL");
    if (!s->have_last) return fail(BHR_ERR_NOT_READY, "bhr_surrogate_trace_stats: no trace yet");
    DevGuard dg(s->device);
    const size_t n = size_t(s->last_nviews);
    const SurrLane& L = s->lane[s->last_lane];
    std::vector<bhr::WorkQueue> q(4 * n + 2);
    int tab_status = 0;
    cudaError_t e = cudaStreamSynchronize(s->last_stream);
    if (e == cudaSuccess) e = cudaMemcpy(q.data(), L.q, sizeof(bhr::WorkQueue) * q.size(), cudaMemcpyDeviceToHost);
    if (e == cudaSuccess)
        e = cudaMemcpy(&tab_status, s->tab_status + s->last_lane, sizeof(int), cudaMemcpyDeviceToHost);
    if (e != cudaSuccess) return cfail(e, "bhr_surrogate_trace_stats");
    if (tab_status)
        return fail(BHR_ERR_TIMEOUT, "bhr_surrogate_trace_stats: a tensor-core completion wait of the table build ran out "
                                     "(the affected table entries are NaN)");
    for (int k = 0; k < 6; ++k) out[k] = 0;
    const bhr::WorkQueue* qb = q.data() + 2 * n + 1;  // the band march's queues
    for (size_t v = 0; v < n; ++v) {
        out[0] += q[2 * v].surr_rays;
        out[1] += q[2 * v].fb_count + qb[2 * v].fb_count;
        out[2] += q[2 * v].capture_disagree;
        out[3] += q[2 * v + 1].steps;
        out[4] += q[2 * v].mlp_queries;
        out[5] += q[2 * v].mlp_rows;
    }
    out[3] += q[2 * n].steps + qb[2 * n].steps;
    // the network runs in the views' tables (whole 128-row tiles)
    out[4] += s->last_rows;
    out[5] += s->last_rows;
    return BHR_OK;
}

}  // extern "C"
