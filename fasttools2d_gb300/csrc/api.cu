// api.cu -- C ABI, context, workspace, FFT plans, parameter selection and the
// driver-level orchestration of the GB300 spectral Ewald library.
#include <cmath>
#include <cstdarg>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <complex>
#include <algorithm>
#include <vector>

#include <atomic>
#include <mutex>
#include <utility>

#include "fte_internal.cuh"
#include "../../include/fasttools2d_debug.h"

// ---------------------------------------------------------------------------
// errors
// ---------------------------------------------------------------------------
static thread_local char g_err[1024] = "";

void fte_set_error(const char* fmt, ...) {
    va_list ap;
    va_start(ap, fmt);
    vsnprintf(g_err, sizeof(g_err), fmt, ap);
    va_end(ap);
}

cudaError_t fte_smem_ceiling_raw(const void* kernel, size_t bytes) {
    static std::mutex mu;
    static std::map<std::pair<int, const void*>, size_t> ceiling;
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) return e;
    std::lock_guard<std::mutex> lock(mu);
    auto key = std::make_pair(dev, kernel);
    auto it = ceiling.find(key);
    if (it == ceiling.end()) {
        int optin = 0;
        e = cudaDeviceGetAttribute(&optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev);
        if (e != cudaSuccess) return e;
        cudaFuncAttributes fa;
        e = cudaFuncGetAttributes(&fa, kernel);
        if (e != cudaSuccess) return e;
        const size_t cap = (size_t)optin > fa.sharedSizeBytes ? (size_t)optin - fa.sharedSizeBytes : 0;
        e = cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)cap);
        if (e != cudaSuccess) return e;
        it = ceiling.emplace(key, cap).first;
    }
    return bytes <= it->second ? cudaSuccess : cudaErrorInvalidValue;
}

// ---------------------------------------------------------------------------
// host-side allocation fault injection (tests)
// ---------------------------------------------------------------------------
static std::atomic<int> g_fail_alloc_countdown{0};

extern "C" int fte_debug_fail_alloc(int after) {
    g_fail_alloc_countdown.store(after > 0 ? after : 0);
    return FTE_OK;
}

bool fte_alloc_should_fail() {
    int v = g_fail_alloc_countdown.load();
    while (v > 0) {
        if (g_fail_alloc_countdown.compare_exchange_weak(v, v - 1)) return v == 1;
    }
    return false;
}

// ---------------------------------------------------------------------------
// input checks
// ---------------------------------------------------------------------------
__global__ void k_count_nonfinite(FiniteSet s, unsigned int* __restrict__ bad) {
    unsigned int cnt = 0;
    for (int a = 0; a < s.k; a++) {
        const double* __restrict__ v = s.p[a];
        for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < s.n[a];
             i += (int64_t)gridDim.x * blockDim.x)
            cnt += isfinite(v[i]) ? 0u : 1u;
    }
    if (cnt) atomicAdd(bad, cnt);
}

int fte_finite_launch(fte_context* c, const FiniteSet& s) {
    unsigned int* host_count = reinterpret_cast<unsigned int*>(c->host_scalars + 48);
    *host_count = 0;
    if (s.k == 0) return FTE_OK;
    int64_t most = 0;
    for (int a = 0; a < s.k; a++) most = s.n[a] > most ? s.n[a] : most;
    int64_t blocks = (most + 255) / 256;
    const int cap = 4 * (c->num_sms > 0 ? c->num_sms : 152);
    const int grid = (int)(blocks < cap ? (blocks < 1 ? 1 : blocks) : cap);
    FTE_CUDA_TRY(cudaMemsetAsync(c->dev_flags, 0, sizeof(unsigned int), c->stream));
    FTE_LAUNCH(c, k_count_nonfinite, grid, 256, 0, s, c->dev_flags);
    FTE_CUDA_TRY(cudaMemcpyAsync(host_count, c->dev_flags, sizeof(unsigned int), cudaMemcpyDeviceToHost, c->stream));
    return FTE_OK;
}

int fte_finite_result(fte_context* c, const char* entry) {
    const unsigned int bad = *reinterpret_cast<const unsigned int*>(c->host_scalars + 48);
    if (bad) {
        fte_set_error("%s: %u non-finite values (NaN or Inf) in the point, density, normal or weight arrays", entry,
                      bad);
        return FTE_ERR_INVALID;
    }
    return FTE_OK;
}

int fte_check_finite(fte_context* c, const FiniteSet& s, const char* entry) {
    if (s.k == 0) return FTE_OK;
    FTE_TRY(fte_finite_launch(c, s));
    FTE_CUDA_TRY(cudaStreamSynchronize(c->stream));
    return fte_finite_result(c, entry);
}

extern "C" const char* fte_last_error(void) { return g_err; }
extern "C" int fte_version(void) { return FTE_VERSION; }

// ---------------------------------------------------------------------------
// context
// ---------------------------------------------------------------------------
extern "C" int fte_create(fte_context** out, int device) {
    if (!out) {
        fte_set_error("fte_create: null output pointer");
        return FTE_ERR_INVALID;
    }
    *out = nullptr;
    int ndev = 0;
    FTE_CUDA_TRY(cudaGetDeviceCount(&ndev));
    if (device < 0 || device >= ndev) {
        fte_set_error("fte_create: device %d not present (%d devices)", device, ndev);
        return FTE_ERR_INVALID;
    }
    FTE_CUDA_TRY(cudaSetDevice(device));
    fte_context* c = new (std::nothrow) fte_context();
    if (!c) {
        fte_set_error("fte_create: out of host memory");
        return FTE_ERR_ALLOC;
    }
    c->device = device;
    cudaDeviceProp prop;
    FTE_CUDA_TRY(cudaGetDeviceProperties(&prop, device));
    c->max_smem_optin = (int)prop.sharedMemPerBlockOptin;
    c->num_sms = prop.multiProcessorCount;
    FTE_CUDA_TRY(cudaStreamCreateWithFlags(&c->own_stream, cudaStreamNonBlocking));
    c->stream = c->own_stream;
    for (int i = 0; i < 8; i++) FTE_CUDA_TRY(cudaEventCreate(&c->ev[i]));
    FTE_CUDA_TRY(cudaEventCreateWithFlags(&c->ev_q, cudaEventDisableTiming));
    FTE_CUDA_TRY(cudaMallocHost(&c->host_scalars, 64 * sizeof(double)));
    FTE_CUDA_TRY(cudaMalloc(&c->dev_flags, 64));
    *out = c;
    return FTE_OK;
}

static void plan_free(FftPlan* p) {
    if (!p) return;
    cudaFree(p->tw);
    cudaFree(p->chirp);
    cudaFree(p->bhat);
    cudaFree(p->tw32);
    cudaFree(p->chirp32);
    cudaFree(p->bhat32);
    cudaFree(p->twff);
    cudaFree(p->chirpff);
    cudaFree(p->bhatff);
    delete p;
}

extern "C" int fte_destroy(fte_context* c) {
    if (!c) return FTE_OK;
    cudaSetDevice(c->device);
    if (c->stream) cudaStreamSynchronize(c->stream);
    for (auto& kv : c->plans) plan_free(kv.second);
    for (auto& kv : c->lplans) {
        cudaFree(kv.second->tw);
        cudaFree(kv.second->chirp);
        cudaFree(kv.second->bhat);
        delete kv.second;
    }
    if (c->ws) cudaFree(c->ws);
    if (c->ws2) cudaFree(c->ws2);
    if (c->host_scalars) cudaFreeHost(c->host_scalars);
    if (c->dev_flags) cudaFree(c->dev_flags);
    for (int i = 0; i < 8; i++)
        if (c->ev[i]) cudaEventDestroy(c->ev[i]);
    if (c->ev_q) cudaEventDestroy(c->ev_q);
    if (c->own_stream) cudaStreamDestroy(c->own_stream);
    delete c;
    return FTE_OK;
}

extern "C" int fte_set_stream(fte_context* c, void* stream) {
    if (!c) {
        fte_set_error("fte_set_stream: null context");
        return FTE_ERR_INVALID;
    }
    c->stream = stream ? (cudaStream_t)stream : c->own_stream;
    return FTE_OK;
}

extern "C" int fte_set_timing(fte_context* c, int enable) {
    if (!c) {
        fte_set_error("fte_set_timing: null context");
        return FTE_ERR_INVALID;
    }
    c->timing = enable ? 1 : 0;
    return FTE_OK;
}

extern "C" long long fte_kernel_count(const fte_context* c) { return c ? c->kernels : 0; }

int fte_ws_reserve(fte_context* c, size_t bytes) {
    if (bytes <= c->ws_size) return FTE_OK;
    if (c->ws) {
        FTE_CUDA_TRY(cudaStreamSynchronize(c->stream));
        cudaFree(c->ws);
        c->ws = nullptr;
        c->ws_size = 0;
    }
    size_t want = bytes + bytes / 8 + (1 << 20);
    cudaError_t e = fte_alloc_should_fail() ? cudaErrorMemoryAllocation : cudaMalloc(&c->ws, want);
    if (e != cudaSuccess) {
        cudaGetLastError();
        fte_set_error("device workspace of %zu bytes could not be allocated: %s", want, cudaGetErrorString(e));
        return FTE_ERR_ALLOC;
    }
    c->ws_size = want;
    return FTE_OK;
}

int fte_ws2_reserve(fte_context* c, size_t bytes) {
    if (bytes <= c->ws2_size) return FTE_OK;
    if (c->ws2) {
        FTE_CUDA_TRY(cudaStreamSynchronize(c->stream));
        cudaFree(c->ws2);
        c->ws2 = nullptr;
        c->ws2_size = 0;
    }
    size_t want = bytes + bytes / 8 + (1 << 20);
    cudaError_t e = fte_alloc_should_fail() ? cudaErrorMemoryAllocation : cudaMalloc(&c->ws2, want);
    if (e != cudaSuccess) {
        cudaGetLastError();
        fte_set_error("device workspace of %zu bytes could not be allocated: %s", want, cudaGetErrorString(e));
        return FTE_ERR_ALLOC;
    }
    c->ws2_size = want;
    return FTE_OK;
}

int fte_record(fte_context* c, int slot) {
    if (!c->timing) return FTE_OK;
    FTE_CUDA_TRY(cudaEventRecord(c->ev[slot], c->stream));
    return FTE_OK;
}

double fte_elapsed(fte_context* c, int a, int b) {
    if (!c->timing) return 0.0;
    float ms = 0.f;
    if (cudaEventElapsedTime(&ms, c->ev[a], c->ev[b]) != cudaSuccess) {
        cudaGetLastError();
        return 0.0;
    }
    return ms;
}

// ---------------------------------------------------------------------------
// FFT plans
// ---------------------------------------------------------------------------
static bool smooth7(int n, std::vector<int>* rad) {
    int v = n;
    int c8 = 0, c2 = 0, c3 = 0, c5 = 0, c7 = 0;
    while (v % 2 == 0) {
        v /= 2;
        c2++;
    }
    while (v % 3 == 0) {
        v /= 3;
        c3++;
    }
    while (v % 5 == 0) {
        v /= 5;
        c5++;
    }
    while (v % 7 == 0) {
        v /= 7;
        c7++;
    }
    if (v != 1) return false;
    if (rad) {
        rad->clear();
        c8 = c2 / 3;
        c2 -= 3 * c8;
        for (int i = 0; i < c8; i++) rad->push_back(8);
        if (c2 == 2) rad->push_back(4);
        if (c2 == 1) rad->push_back(2);
        for (int i = 0; i < c3; i++) rad->push_back(3);
        for (int i = 0; i < c5; i++) rad->push_back(5);
        for (int i = 0; i < c7; i++) rad->push_back(7);
    }
    return true;
}

// exp(-2 pi i num/den) with the numerator reduced first
static std::complex<double> unit_root(long long num, long long den) {
    num %= den;
    if (num < 0) num += den;
    double ang;
    if (2 * num <= den)
        ang = -2.0 * FTE_PI * (double)num / (double)den;
    else
        ang = 2.0 * FTE_PI * (double)(den - num) / (double)den;
    return {std::cos(ang), std::sin(ang)};
}

// host recursive mixed-radix DFT (for the Bluestein kernel only)
static void host_dft(std::vector<std::complex<double>>& a) {
    size_t n = a.size();
    if (n <= 1) return;
    size_t p = 0;
    for (size_t q : {2, 3, 5, 7})
        if (n % q == 0) {
            p = q;
            break;
        }
    if (p == 0) {
        std::vector<std::complex<double>> o(n);
        for (size_t k = 0; k < n; k++) {
            std::complex<double> s = 0;
            for (size_t j = 0; j < n; j++) s += a[j] * unit_root((long long)(j * k % n), (long long)n);
            o[k] = s;
        }
        a = o;
        return;
    }
    size_t m = n / p;
    std::vector<std::vector<std::complex<double>>> sub(p, std::vector<std::complex<double>>(m));
    for (size_t q = 0; q < p; q++)
        for (size_t j = 0; j < m; j++) sub[q][j] = a[j * p + q];
    for (size_t q = 0; q < p; q++) host_dft(sub[q]);
    for (size_t k = 0; k < n; k++) {
        std::complex<double> s = 0;
        for (size_t q = 0; q < p; q++) s += sub[q][k % m] * unit_root((long long)(q * k % n), (long long)n);
        a[k] = s;
    }
}

// float-float copy of a complex FP64 value
static float4 ff4(std::complex<double> z) {
    const float rh = (float)z.real(), ih = (float)z.imag();
    return make_float4(rh, (float)(z.real() - (double)rh), ih, (float)(z.imag() - (double)ih));
}

template <typename T>
static int upload(T** dst, const std::vector<T>& v) {
    FTE_CUDA_TRY(cudaMalloc(dst, v.size() * sizeof(T)));
    FTE_CUDA_TRY(cudaMemcpy(*dst, v.data(), v.size() * sizeof(T), cudaMemcpyHostToDevice));
    return FTE_OK;
}

int fte_get_plan(fte_context* c, int n, FftDev* out) {
    auto it = c->plans.find(n);
    FftPlan* p = nullptr;
    if (it != c->plans.end()) {
        p = it->second;
    } else {
        p = new FftPlan();
        p->n = n;
        std::vector<int> rad;
        if (smooth7(n, &rad)) {
            p->m = n;
        } else {
            p->bluestein = 1;
            int m = 2 * n - 1;
            while (!smooth7(m, nullptr)) m++;
            smooth7(m, &rad);
            p->m = m;
        }
        if (rad.size() > 24) {
            delete p;
            fte_set_error("FFT length %d has too many factors", n);
            return FTE_ERR_UNSUPPORTED;
        }
        p->nrad = (int)rad.size();
        for (size_t i = 0; i < rad.size(); i++) p->rad[i] = rad[i];
        const int m = p->m;
        std::vector<double2> tw(m);
        std::vector<float2> tw32(m);
        std::vector<float4> twf(m);
        for (int t = 0; t < m; t++) {
            auto z = unit_root(t, m);
            tw[t] = make_double2(z.real(), z.imag());
            tw32[t] = make_float2((float)z.real(), (float)z.imag());
            twf[t] = ff4(z);
        }
        int st = upload(&p->tw, tw);
        if (!st) st = upload(&p->tw32, tw32);
        if (!st) st = upload(&p->twff, twf);
        if (!st && p->bluestein) {
            std::vector<double2> ch(n);
            std::vector<float2> ch32(n);
            std::vector<float4> chf(n);
            std::vector<std::complex<double>> b(m, 0.0);
            for (int k = 0; k < n; k++) {
                long long k2 = ((long long)k * k) % (2LL * n);
                auto z = unit_root(k2, 2LL * n);  // exp(-i pi k^2 / n)
                ch[k] = make_double2(z.real(), z.imag());
                ch32[k] = make_float2((float)z.real(), (float)z.imag());
                chf[k] = ff4(z);
                b[k] = std::conj(z);
                if (k > 0) b[m - k] = std::conj(z);
            }
            host_dft(b);
            std::vector<double2> bh(m);
            std::vector<float2> bh32(m);
            std::vector<float4> bhf(m);
            for (int k = 0; k < m; k++) {
                auto z = b[k] / (double)m;
                bh[k] = make_double2(z.real(), z.imag());
                bh32[k] = make_float2((float)z.real(), (float)z.imag());
                bhf[k] = ff4(z);
            }
            st = upload(&p->chirp, ch);
            if (!st) st = upload(&p->chirp32, ch32);
            if (!st) st = upload(&p->bhat, bh);
            if (!st) st = upload(&p->bhat32, bh32);
            if (!st) st = upload(&p->chirpff, chf);
            if (!st) st = upload(&p->bhatff, bhf);
        }
        if (st) {
            plan_free(p);
            return st;
        }
        c->plans[n] = p;
    }
    out->n = p->n;
    out->m = p->m;
    out->nrad = p->nrad;
    out->bluestein = p->bluestein;
    for (int i = 0; i < 24; i++) out->rad[i] = p->rad[i];
    out->tw = p->tw;
    out->chirp = p->chirp;
    out->bhat = p->bhat;
    out->tw32 = p->tw32;
    out->chirp32 = p->chirp32;
    out->bhat32 = p->bhat32;
    out->twff = p->twff;
    out->chirpff = p->chirpff;
    out->bhatff = p->bhatff;
    return FTE_OK;
}

// ---- long transforms -----------------------------------------------------------
// inner length of the block transform of n: n when 7-smooth, else the
// Bluestein length (smallest 7-smooth m >= 2n - 1)
static long long block_inner(int n) {
    std::vector<int> rad;
    if (smooth7(n, &rad)) return rad.size() <= 24 ? n : -1;
    long long m = 2LL * n - 1;
    while (!smooth7((int)m, nullptr)) m++;
    return m;
}

bool fte_fft_fits_block(int n, int complex_bytes) {
    if (n < 1) return false;
    long long m = block_inner(n);
    return m > 0 && 2 * m * complex_bytes <= kFftSmemCap;
}

// L = n1 * n2 with both factors block-transformable in FP64: prefer 7-smooth
// factors (no in-block Bluestein), then the most balanced split.
static bool split_factors(int L, bool smooth_only, int* n1, int* n2) {
    int best = 0;
    for (int a = 2; (long long)a * a <= L; a++) {
        if (L % a) continue;
        int b = L / a;
        if (smooth_only && !(smooth7(a, nullptr) && smooth7(b, nullptr))) continue;
        if (!fte_fft_fits_block(a, 16) || !fte_fft_fits_block(b, 16)) continue;
        best = a;  // increasing a: the last fit is the most balanced
    }
    if (!best) return false;
    // the contiguous second pass transforms n1: give it the larger factor
    *n1 = L / best;
    *n2 = best;
    return true;
}

bool fte_long_shape(int n, int* mode, int* L, int* n1, int* n2) {
    if (n < 4) return false;
    if (split_factors(n, true, n1, n2) || split_factors(n, false, n1, n2)) {
        *mode = 1;
        *L = n;
        return true;
    }
    for (long long m = 2LL * n - 1; m < (1LL << 30); m++) {
        if (!smooth7((int)m, nullptr)) continue;
        if (split_factors((int)m, true, n1, n2)) {
            *mode = 2;
            *L = (int)m;
            return true;
        }
    }
    return false;
}

size_t fte_long_scratch(int n, long long nl) {
    int mode, L, n1, n2;
    if (!fte_long_shape(n, &mode, &L, &n1, &n2)) return 0;
    return (size_t)(mode == 1 ? 1 : 2) * (size_t)nl * (size_t)L;
}

int fte_get_long_plan(fte_context* c, int n, LongFft* out) {
    auto it = c->lplans.find(n);
    if (it != c->lplans.end()) {
        *out = it->second->dev;
        return FTE_OK;
    }
    int mode, L, n1, n2;
    if (!fte_long_shape(n, &mode, &L, &n1, &n2)) {
        fte_set_error("FFT length %d: no block factorisation", n);
        return FTE_ERR_UNSUPPORTED;
    }
    LongPlan* p = new LongPlan();
    p->dev.n = n;
    p->dev.mode = mode;
    p->dev.L = L;
    p->dev.n1 = n1;
    p->dev.n2 = n2;
    int st = fte_get_plan(c, n1, &p->dev.d1);
    if (!st) st = fte_get_plan(c, n2, &p->dev.d2);
    std::vector<double2> tw(L);
    for (int t = 0; t < L; t++) {
        auto z = unit_root(t, L);
        tw[t] = make_double2(z.real(), z.imag());
    }
    if (!st) st = upload(&p->tw, tw);
    if (!st && mode == 2) {
        std::vector<double2> ch(n);
        std::vector<std::complex<double>> b(L, 0.0);
        for (int k = 0; k < n; k++) {
            long long k2 = ((long long)k * k) % (2LL * n);
            auto z = unit_root(k2, 2LL * n);  // exp(-i pi k^2 / n)
            ch[k] = make_double2(z.real(), z.imag());
            b[k] = std::conj(z);
            if (k > 0) b[L - k] = std::conj(z);
        }
        host_dft(b);
        std::vector<double2> bh(L);
        for (int k = 0; k < L; k++) {
            auto z = b[k] / (double)L;
            bh[k] = make_double2(z.real(), z.imag());
        }
        st = upload(&p->chirp, ch);
        if (!st) st = upload(&p->bhat, bh);
    }
    if (st) {
        cudaFree(p->tw);
        cudaFree(p->chirp);
        cudaFree(p->bhat);
        delete p;
        return st;
    }
    p->dev.tw = p->tw;
    p->dev.chirp = p->chirp;
    p->dev.bhat = p->bhat;
    c->lplans[n] = p;
    *out = p->dev;
    return FTE_OK;
}

int fte_fft_prepare(fte_context* c, int n) {
    if (fte_fft_fits_block(n, 16)) {
        FftDev d;
        return fte_get_plan(c, n, &d);
    }
    LongFft f;
    return fte_get_long_plan(c, n, &f);
}

// ---------------------------------------------------------------------------
// parameter selection: the MATLAB drivers' analytic choice
// (StokesSLP_ewald_2p.m:27-35,85-104 and find_kinfb :147-173, find_xi :178-202;
//  StokesDLP_ewald_2p.m:27-38,105-125 and find_kinfb :171-197, find_xi :202-224).
// Estimates of Palsson & Tornberg 2019; Newton iterations with the step in
// the negative direction limited to 0.9 of the iterate, at most 101 steps.
// find_kinfb is called with Lx in place of Ly, as the drivers do.
// ---------------------------------------------------------------------------
namespace {

// MATLAB rat with tolerance 1e-6 |x| (nearest-integer continued fraction)
void matlab_rat(double x, int* num, int* den) {
    double tol = 1e-6 * std::fabs(x);
    double lastn = 1, lastd = 0, n = std::round(x), d = 1, frac = x - n;
    for (int guard = 0; std::fabs(x - n / d) >= tol && guard < 64; guard++) {
        double flip = 1 / frac, step = std::round(flip);
        frac = flip - step;
        double sn = n;
        n = n * step + lastn;
        lastn = sn;
        double sd = d;
        d = d * step + lastd;
        lastd = sd;
    }
    *num = (int)(n * (d > 0 ? 1 : (d < 0 ? -1 : 0)));
    *den = (int)std::fabs(d);
}

template <typename F, typename FP>
double newton(double x, double tol, F f, FP fp) {
    for (int it = 0;; it++) {
        double fx = f(x);
        if (!(std::fabs(fx) > tol)) break;
        if (it > 100) break;
        double d = fx / fp(x);
        if (0.9 * x < d) d = 0.9 * x;
        x -= d;
    }
    return x;
}

int matlab_length(int64_t n) { return n == 0 ? 0 : (n > 2 ? (int)n : 2); }

}  // namespace

static int choose_params_q(int kind, int64_t nsrc, int64_t ntar, double Q, double Lx, double Ly,
                           const fte_options* opt, fte_params* o) {
    std::memset(o, 0, sizeof(*o));
    int P = (opt && opt->P > 0) ? opt->P : 24;
    double tol = (opt && opt->tol > 0) ? opt->tol : 1e-16;
    double npts = (double)nsrc + (double)ntar;
    double Nb = (opt && opt->Nb > 0) ? opt->Nb : std::fmin(P * std::round(std::log2(npts)), npts / 4);
    int A, B;
    matlab_rat(Lx / Ly, &A, &B);
    if (A <= 0 || B <= 0) {
        fte_set_error("box aspect ratio Lx/Ly = %g has no usable rational approximation", Lx / Ly);
        return FTE_ERR_INVALID;
    }
    if (kind == FTE_KIND_DLP) npts = (double)matlab_length(nsrc) + (double)matlab_length(ntar);
    int a = (int)std::ceil(std::sqrt(npts / (Nb * A * B)));
    if (a < 1) a = 1;
    const double m = 0.95 * std::sqrt(FTE_PI * P);
    o->P = P;
    o->Nb = Nb;
    o->tol = tol;
    o->Q = Q;
    o->A = A;
    o->B = B;
    o->nside_x = (opt && opt->nside_x > 0) ? opt->nside_x : a * A;
    o->nside_y = (opt && opt->nside_y > 0) ? opt->nside_y : a * B;
    double rc = Lx / o->nside_x;
    o->rc = rc;
    double xi;
    if (opt && opt->xi > 0) {
        xi = opt->xi;
    } else if (kind == FTE_KIND_SLP) {
        xi = newton(
            4 / rc, tol,
            [&](double x) { return std::sqrt(Q * FTE_PI / (4 * Lx * Ly * x)) * std::exp(-x * x * rc * rc) - tol; },
            [&](double x) {
                return -std::sqrt(Q * FTE_PI / (4 * Lx * Ly)) * std::exp(-x * x * rc * rc) *
                       (0.5 * std::pow(x, -1.5) + 2 * rc * rc * x * std::sqrt(1 / x));
            });
    } else {
        xi = newton(
            1 / rc, tol,
            [&](double x) { return std::exp(-x * x * rc * rc) * x * rc * std::sqrt(2 * FTE_PI * Q / (Lx * Ly)) - tol; },
            [&](double x) {
                return (1 - 2 * x * x * rc * rc) * std::exp(-x * x * rc * rc) * std::sqrt(2 * FTE_PI * Q / (Lx * Ly)) * rc;
            });
    }
    o->xi = xi;
    const double L1 = Lx, L2 = Lx;  // find_kinfb(Q, Lx, Lx, xi, tol)
    const double mx = L1 > L2 ? L1 : L2;
    double k;
    if (kind == FTE_KIND_SLP) {
        k = newton(
            std::round(5 * xi), tol,
            [&](double k) {
                return std::sqrt(4 * Q * FTE_PI * mx / (L1 * L1 * L1 * L2 * L2 * L2 * k)) * std::exp(-k * k / (4 * xi * xi)) - tol;
            },
            [&](double k) {
                return -std::sqrt(4 * Q * FTE_PI * mx / (L1 * L1 * L1 * L2 * L2 * L2)) * std::exp(-k * k / (4 * xi * xi)) *
                       (0.5 * std::pow(k, -1.5) + std::sqrt(1 / k) * 2 * k / (4 * xi * xi));
            });
    } else {
        // left-to-right as in MATLAB: k*8*pi*Q*max(Lx,Ly)/Lx^3*Ly^3
        k = newton(
            std::round(5 * xi), tol,
            [&](double k) {
                return std::sqrt(k * 8 * FTE_PI * Q * mx / (L1 * L1 * L1) * (L2 * L2 * L2)) * std::exp(-k * k / (4 * xi * xi)) - tol;
            },
            [&](double k) {
                return std::sqrt(8 * FTE_PI * Q * mx / (L1 * L1 * L1) * (L2 * L2 * L2)) * std::exp(-k * k / (4 * xi * xi)) *
                       (0.5 * std::pow(k, -0.5) - 2 * std::pow(k, 1.5) / (4 * xi * xi));
            });
    }
    int kinf = (int)std::round(Lx * k / (2 * FTE_PI));
    o->kinf = kinf;
    int M = 2 * kinf < 10000 ? 2 * kinf : 10000;
    o->Mx = (opt && opt->Mx > 0) ? opt->Mx : A * M;
    o->My = (opt && opt->My > 0) ? opt->My : B * M;
    o->w = P * Lx / o->Mx / 2;
    o->eta = (2 * xi * o->w / m) * (2 * xi * o->w / m);
    return FTE_OK;
}

// ---------------------------------------------------------------------------
// Tuned parameters of the mixed form.  The analytic estimates above are kept
// (the same Newton solves for xi and kinf), but every free choice the drivers
// fix is optimised for speed at the requested tolerance:
//   * P: smallest even support whose window error erfc(m/sqrt 2),
//     m = 0.95 sqrt(pi P), is below tol/300 (the drivers always use 24; the
//     measured window error of the stresslet k-space part is ~50-100 x this
//     term relative to max |u|);
//   * the cell multiplier a (cutoff rc = Lx/(a A)): minimises a cost model of
//     near pairs (FP64), window work (spread + gather) and FFTs, with unit
//     costs measured on GB300; the drivers take a from Nb;
//   * grids rounded up to 7-smooth even sizes (no Bluestein transform);
//   * the k-space part in FP32 when tol >= 1e-7, else in FP64;
//   * the estimates are solved for tol * slack: they bound the error by
//     sum |f|^2, which over-estimates the max-relative error of the result by
//     one to three orders of magnitude on the benchmark inputs (least for
//     the stresslet at small N); slack = 3.
// ---------------------------------------------------------------------------
namespace {

// x0, k0 > 0: start the Newton iteration there instead of the drivers' start
// (the tuned chooser starts each candidate from the previous one's root)
double xi_estimate(int kind, double Q, double Lx, double Ly, double rc, double tol, double x0 = 0) {
    if (kind == FTE_KIND_SLP)
        return newton(
            x0 > 0 ? x0 : 4 / rc, tol,
            [&](double x) { return std::sqrt(Q * FTE_PI / (4 * Lx * Ly * x)) * std::exp(-x * x * rc * rc) - tol; },
            [&](double x) {
                return -std::sqrt(Q * FTE_PI / (4 * Lx * Ly)) * std::exp(-x * x * rc * rc) *
                       (0.5 * std::pow(x, -1.5) + 2 * rc * rc * x * std::sqrt(1 / x));
            });
    return newton(
        x0 > 0 ? x0 : 1 / rc, tol,
        [&](double x) { return std::exp(-x * x * rc * rc) * x * rc * std::sqrt(2 * FTE_PI * Q / (Lx * Ly)) - tol; },
        [&](double x) {
            return (1 - 2 * x * x * rc * rc) * std::exp(-x * x * rc * rc) * std::sqrt(2 * FTE_PI * Q / (Lx * Ly)) * rc;
        });
}

double kinf_root(int kind, double Q, double Lx, double xi, double tol, double k0 = 0) {
    const double L1 = Lx;
    double k;
    if (kind == FTE_KIND_SLP)
        k = newton(
            k0 > 0 ? k0 : std::round(5 * xi), tol,
            [&](double k) {
                return std::sqrt(4 * Q * FTE_PI * L1 / (std::pow(L1, 6) * k)) * std::exp(-k * k / (4 * xi * xi)) - tol;
            },
            [&](double k) {
                return -std::sqrt(4 * Q * FTE_PI * L1 / std::pow(L1, 6)) * std::exp(-k * k / (4 * xi * xi)) *
                       (0.5 * std::pow(k, -1.5) + std::sqrt(1 / k) * 2 * k / (4 * xi * xi));
            });
    else
        k = newton(
            k0 > 0 ? k0 : std::round(5 * xi), tol,
            [&](double k) { return std::sqrt(k * 8 * FTE_PI * Q * L1) * std::exp(-k * k / (4 * xi * xi)) - tol; },
            [&](double k) {
                return std::sqrt(8 * FTE_PI * Q * L1) * std::exp(-k * k / (4 * xi * xi)) *
                       (0.5 * std::pow(k, -0.5) - 2 * std::pow(k, 1.5) / (4 * xi * xi));
            });
    return k;
}
// transform work of a length-n line relative to a 7-smooth line of n points:
// Bluestein runs two transforms of a smooth length m >= 2n - 1 (about 2.2 n)
// Transform work per point of a length-n line: the sum over the Stockham
// passes of each radix's arithmetic per point (twiddles included; radix 8
// does three levels for 9 FP64 operations per point, the paired odd-radix
// DFTs cost more per level); Bluestein runs two transforms of a smooth
// length m >= 2n - 1 plus the chirp products.
// per-point cost of the Stockham passes of a 7-smooth n (radix-8 passes
// first, then one 4 or 2, then 3, 5, 7 as the plans order them); -1 when n
// is not 7-smooth.  Allocation-free: the chooser calls it thousands of times.
double smooth_line_cost(int n) {
    if (n < 1) return -1;
    int c2 = 0, c3 = 0, c5 = 0, c7 = 0;
    while (n % 2 == 0) n /= 2, c2++;
    while (n % 3 == 0) n /= 3, c3++;
    while (n % 5 == 0) n /= 5, c5++;
    while (n % 7 == 0) n /= 7, c7++;
    if (n != 1) return -1;
    const int c8 = c2 / 3, r2 = c2 - 3 * c8;
    return 9.0 * c8 + (r2 == 2 ? 7.0 : (r2 == 1 ? 5.0 : 0.0)) + 8.0 * c3 + 11.0 * c5 + 13.0 * c7;
}
double line_cost_direct(int n) {
    const double c = smooth_line_cost(n);
    if (c >= 0) return c;
    // Bluestein: two transforms of a smooth length near 2n plus the chirp
    // products, per point of n (estimated without searching the length)
    const double m = 2.2 * n;
    return (2 * 3.4 * std::log2(m) + 12) * m / n;
}
// line_cost for lengths below 32768 from a table built once per process (the
// tuned chooser evaluates it ~10^4 times per call while the GPU waits)
double line_cost(int n) {
    constexpr int kMax = 32768;
    static const std::vector<double> tab = [] {
        std::vector<double> t(kMax);
        for (int i = 1; i < kMax; i++) t[i] = line_cost_direct(i);
        return t;
    }();
    return n > 0 && n < kMax ? tab[n] : line_cost_direct(n);
}
// 2-D transform work of an Mx x My grid in units that equal points x log2(points)
// for power-of-two sides (about 3.1 operations per point and level)
double fft_work(int Mx, int My) { return (double)Mx * My * (line_cost(Mx) + line_cost(My)) / 3.1; }

// Grid resolving kinf modes along Lx with square cells (hx = hy):
// Mx = A t, My = B t (Lx / Ly = A / B), t >= 2 kinf / A, both even; among
// the t in a short range the one with the least transform work.  (The
// drivers use Mx = A * 2 kinf, which over-resolves by A along each side.)
void pick_grid(int A, int B, int kinf, int* Mx, int* My) {
    int t0 = (int)std::ceil(2.0 * kinf / A);
    if (t0 < 2) t0 = 2;
    double best = 1e300;
    int bt = t0;
    int span = t0 / 8 > 16 ? t0 / 8 : 16;
    if (span > 128) span = 128;
    for (int t = t0; t <= t0 + span; t++) {
        int mx = A * t, my = B * t;
        if (mx % 2 || my % 2) continue;
        double w = fft_work(mx, my);
        if (w < best) {
            best = w;
            bt = t;
        }
    }
    if (A * bt % 2 || B * bt % 2) bt += 1;
    *Mx = A * bt;
    *My = B * bt;
}

// Grid with its own step per axis (boxes whose aspect ratio is no small
// rational): each side resolves the same wave number, Mx >= 2 kx, My >= 2 ky
// (kx = Lx k / 2 pi, ky = Ly k / 2 pi), both even; among the even sizes up to
// a short span above those bounds, the pair with the least transform work.
void pick_grid_axes(double kx, double ky, int* Mx, int* My) {
    auto lo = [](double k) {
        int m = (int)std::ceil(2.0 * k - 1e-9);
        if (m < 2) m = 2;
        return m + (m & 1);
    };
    const int x0 = lo(kx), y0 = lo(ky);
    auto span = [](int m) {
        int s = m / 8 > 16 ? m / 8 : 16;
        return s > 128 ? 128 : s;
    };
    double best = 1e300;
    int bx = x0, by = y0;
    for (int mx = x0; mx <= x0 + span(x0); mx += 2) {
        const double cx = line_cost(mx);
        for (int my = y0; my <= y0 + span(y0); my += 2) {
            const double w = (double)mx * my * (cx + line_cost(my));
            if (w < best) {
                best = w;
                bx = mx;
                by = my;
            }
        }
    }
    *Mx = bx;
    *My = by;
}

}  // namespace

// Unit costs (seconds) of the cost model, fitted on GB300 to stage times of
// the mixed form at 1e6 uniform points, tolerances 1e-10, 1e-8 and 1e-6,
// cell lists of 100^2 to 225^2 boxes: the near field as per-target +
// per-pair + per-box terms (the box term is the staging of each 3x3
// neighbourhood and the drain of the pair queues at each box's end), spread
// + gather per window node and grid, transforms per unit of fft_work.
static const double kCostTarget = 0.3e-9;      // near field, per target
static const double kCostPair = 14e-12;        // per pair within the cutoff (float-float / FP32 classes)
static const double kCostPair64 = 40e-12;      // same with FP64 pairs (tolerances below 1e-11)
static const double kCostBox = 28e-9;          // per box of the cell list
static const double kCostWin64 = 3.2e-12;      // one window node x grid, FP64 spread/gather
static const double kCostWin32 = 2.5e-12;      // same in FP32 (an exponential per node)
static const double kCostWinFF = 1.31e-12;     // same in float-float (FP32 pipe), window records included
static const double kCostWinFS = 0.83e-12;     // same with FP32 products and compensated sums (FTE_FORM_FF32)
static const double kCostGridFF = 16e-12;      // float-float: per grid node x grid (tile staging, flushes)
static const double kCostFft64 = 9e-12;        // per unit of fft_work, 7-smooth FP64 block transforms
static const double kCostFftFF = 2.3e-12;      // same in float-float (filter included)
static const double kCostFft32 = 3e-12;        // same in FP32
// Calibration of the tuned choice against converged FP64 sums on 2000
// generated configurations (uniform and clustered points, aspect 1..4,
// tolerances 1e-12..1e-4): the stresslet's estimates meet the tolerance with
// slack 3 and the window rule erfc(m / sqrt 2) <= tol / 300, the Stokeslet
// needs no slack and one more window step (tol / 3000), and FP32 grids bottom
// out near 2.5e-7 (Stokeslet) and 4e-8 (stresslet) relative.
static const double kTolSlack[2] = {1.0, 3.0};
// The k-space truncation of the Stokeslet estimate is an RMS figure for
// spread-out sources: at targets on densely sampled boundaries (sources
// 1e-3 apart on curves, config 2's ellipses in a 2 x 1 box) the max-norm
// error reached 3x the tolerance at the estimate's kinf.  kinf is therefore
// taken at the tolerance times this factor (the grid grows ~4 % per side).
static const double kKinfSlack[2] = {0.1, 1.0};
static const double kWinRatio[2] = {3000.0, 300.0};
// (also the floor of FTE_FORM_FF32: its FP32 products left 1.6e-7 / 1.6e-8
// at 1e6 uniform points on the parameters of tol 1e-11)
static const double kFp32Floor[2] = {1e-6, 2e-7};
// FTE_FORM_FF32 only up to this window support: measured at 6000 points
// against FP64 on the same parameters, the k-space part stays at the FP32
// floor (~1e-7) up to P = 36 and then loses accuracy in the Stokeslet spread
// (5e-6 at P = 40, 5e-3 at P = 44); the float-float spread with the FP32
// gather stays at the floor there, the FP32-product spread is the part that
// degrades.  The tuned choice reaches FTE_FORM_FF32 at P <= 16.
static const int kFf32MaxP = 30;
// float-float spread and gather (~48-bit values) hold their ~1e-13 relative
// error well below tolerances from 1e-11 up
static const double kFfFloor[2] = {1e-11, 1e-11};

static int choose_params_tuned(int kind, int64_t nsrc, int64_t ntar, double Q, double Lx, double Ly,
                               const fte_options* opt, fte_params* o) {
    // start from the analytic choice (Nb, rat, defaults) and re-optimise
    FTE_TRY(choose_params_q(kind, nsrc, ntar, Q, Lx, Ly, opt, o));
    const double tol = o->tol;
    const double tol_e = tol * (opt && opt->slack > 0 ? opt->slack : kTolSlack[kind]);
    const int force = opt ? opt->kspace : FTE_KSPACE_AUTO;
    if (force < FTE_KSPACE_AUTO || force > FTE_KSPACE_FF32) {
        fte_set_error("unknown k-space arithmetic %d", force);
        return FTE_ERR_INVALID;
    }
    if (force == FTE_KSPACE_FF32 && opt && opt->P > kFf32MaxP) {
        fte_set_error("FP32-product k-space: window support P=%d above %d (its Stokeslet spread loses accuracy "
                      "beyond that)", opt->P, kFf32MaxP);
        return FTE_ERR_UNSUPPORTED;
    }
    const bool fp32 = tol >= kFp32Floor[kind];
    const bool ffok = tol >= kFfFloor[kind];
    int P = opt && opt->P > 0 ? opt->P : 0;
    if (P == 0) {
        for (P = 4; P < 24; P += 2) {
            double m = 0.95 * std::sqrt(FTE_PI * P);
            if (std::erfc(m / std::sqrt(2.0)) <= tol / kWinRatio[kind]) break;
        }
    }
    const int A = o->A, B = o->B;
    // A box whose aspect ratio is a small rational A / B keeps the drivers'
    // geometry: square cells (nside = a (A, B)) and equal grid steps
    // (M = t (A, B)).  Any other box -- Lx / Ly irrational, or a ratio whose
    // rat() terms are large, for which the drivers' cell list and A-fold grid
    // explode -- gets cells of nearly equal sides (Lx / rc0 and Ly / rc0
    // rounded; the cutoff is the shorter side) and a grid step per axis.
    const bool rational = A <= 16 && B <= 16 && std::fabs(Lx * B - Ly * A) <= 1e-12 * Lx * B;
    const int a0 = o->nside_x / A;
    // cells holding the drivers' Nb points on average
    const double rc_ref = std::sqrt(Lx * Ly * o->Nb / std::fmax(1.0, (double)nsrc + (double)ntar));
    int last_nsx = -1, last_nsy = -1;
    const double area = Lx * Ly;
    const int ng = kind == FTE_KIND_SLP ? 2 : 4;
    const double nfft = kind == FTE_KIND_SLP ? 2.0 : 3.0;
    double best = 1e300;
    fte_params bestp = *o;
    int best_form = FTE_FORM_PLAIN;
    int last_a = -1;
    // Newton roots of the previous candidate (warm starts: the estimates'
    // roots scale about as 1 / rc and xi, and a cold start from the drivers'
    // guess takes tens of iterations per candidate)
    double prev_xr = 0, prev_k = 0, prev_xi = 0;
    for (int step = -12; step <= 40; step++) {
        int nsx, nsy;
        if (rational) {
            int a = (int)std::lround(a0 * std::pow(1.1, step));
            if (opt && opt->nside_x > 0) a = opt->nside_x / A;
            if (a < 1 || a == last_a) continue;
            last_a = a;
            nsx = a * A;
            nsy = a * B;
        } else {
            const double rc0 = rc_ref * std::pow(1.1, -step);
            nsx = (int)std::lround(Lx / rc0);
            nsy = (int)std::lround(Ly / rc0);
            if (opt && opt->nside_x > 0) {
                nsx = opt->nside_x;
                nsy = opt->nside_y > 0 ? opt->nside_y : (int)std::lround(Ly * nsx / Lx);
            }
            if (nsx < 1) nsx = 1;
            if (nsy < 1) nsy = 1;
            if ((nsx == last_nsx && nsy == last_nsy) || (double)nsx * nsy > 1e8) continue;
            last_nsx = nsx;
            last_nsy = nsy;
        }
        double rc = rational ? Lx / nsx : std::fmin(Lx / nsx, Ly / nsy);
        // (10 % below the scaled root: the iteration then enters the
        // convergence band from the same side as from the drivers' start)
        double xi = (opt && opt->xi > 0) ? opt->xi : xi_estimate(kind, Q, Lx, Ly, rc, tol_e, 0.9 * prev_xr / rc);
        const double kr =
            kinf_root(kind, Q, Lx, xi, tol_e * kKinfSlack[kind], prev_xi > 0 ? 0.9 * prev_k * xi / prev_xi : 0);
        prev_xr = xi * rc;
        prev_k = kr;
        prev_xi = xi;
        int kinf = (int)std::round(Lx * kr / (2 * FTE_PI));
        int Mx, My;
        if (rational)
            pick_grid(A, B, kinf, &Mx, &My);
        else
            pick_grid_axes(Lx * kr / (2 * FTE_PI), Ly * kr / (2 * FTE_PI), &Mx, &My);
        if (opt && opt->Mx > 0) Mx = opt->Mx;
        if (opt && opt->My > 0) My = opt->My;
        if (rational && std::fabs(Lx / Mx - Ly / My) > 1e-12 * (Lx / Mx)) continue;
        if ((double)Mx * My > 4.0e8) continue;  // 4 grids of 4e8 nodes: 13 GB
        if (P + 1 > Mx || P + 1 > My) continue;
        // k-space arithmetic: the cheapest the tolerance allows (FP32 only
        // with block transforms) unless forced; FP64 lines longer than a
        // block take the long transform, and so do the float-float form's
        const bool fits32 = fte_fft_fits_block(Mx, 8) && fte_fft_fits_block(My, 8);
        const bool long64 = !fte_fft_fits_block(Mx, 16) || !fte_fft_fits_block(My, 16);
        const double pairs = (double)nsrc * (double)ntar * FTE_PI * rc * rc / area * 1.03;
        const double win = (double)(P + 1) * (P + 1) * ((double)nsrc * ng + (double)ntar * 2);
        const double fftw = fft_work(Mx, My) * nfft;
        // the float-float stresslet spreads and transforms three grids
        // (the symmetric products), not four
        const double winff = kind == FTE_KIND_SLP ? win : (double)(P + 1) * (P + 1) * ((double)nsrc * 3 + (double)ntar * 2);
        const double fftwff = kind == FTE_KIND_SLP ? fftw : fft_work(Mx, My) * 2.5;
        const double near = kCostTarget * (double)ntar + (ffok ? kCostPair : kCostPair64) * pairs +
                            kCostBox * (double)nsx * (double)nsy;
        int kf = -1;
        double cost = 1e300;
        for (int f : {FTE_FORM_MIXED, FTE_FORM_FF32, FTE_FORM_FF, FTE_FORM_PLAIN}) {
            bool allowed;
            if (force == FTE_KSPACE_AUTO)
                allowed = f == FTE_FORM_MIXED ? fp32 && fits32
                                              : (f == FTE_FORM_FF32 ? fp32 && ffok && P <= kFf32MaxP
                                                                    : (f == FTE_FORM_FF ? ffok : true));
            else if (force == FTE_KSPACE_FP32)
                allowed = f == FTE_FORM_MIXED && fits32;
            else
                allowed = f == (force == FTE_KSPACE_FF     ? FTE_FORM_FF
                                : force == FTE_KSPACE_FF32 ? FTE_FORM_FF32
                                                           : FTE_FORM_PLAIN);
            if (!allowed) continue;
            double c;
            if (f == FTE_FORM_MIXED)
                c = kCostWin32 * win + kCostFft32 * fftw;
            else if (fte_form_ff(f))
                c = (f == FTE_FORM_FF32 ? kCostWinFS : kCostWinFF) * winff +
                    kCostGridFF * (double)Mx * My * (kind == FTE_KIND_SLP ? 4 : 5) +
                    (long64 ? 2.5 * kCostFft64 : kCostFftFF) * fftwff;
            else
                c = kCostWin64 * win + (long64 ? 2.5 : 1.0) * kCostFft64 * fftw;
            if (c < cost) {
                cost = c;
                kf = f;
            }
        }
        if (kf < 0) continue;
        cost += near;
        if (cost < best) {
            best = cost;
            bestp = *o;
            bestp.P = P;
            bestp.nside_x = nsx;
            bestp.nside_y = nsy;
            bestp.rc = rc;
            bestp.xi = xi;
            bestp.kinf = kinf;
            bestp.Mx = Mx;
            bestp.My = My;
            double m = 0.95 * std::sqrt(FTE_PI * P);
            bestp.w = P * Lx / Mx / 2;
            // one Gaussian shape for both axes, set by the narrower support
            const double wmin = rational ? bestp.w : P * std::fmin(Lx / Mx, Ly / My) / 2;
            bestp.eta = (2 * xi * wmin / m) * (2 * xi * wmin / m);
            best_form = kf;
        }
        if (opt && opt->nside_x > 0) break;
    }
    (void)last_a;
    if (best >= 1e300) {
        fte_set_error("no tuned parameters within the grid limits (%d x %d boxes)", o->nside_x, o->nside_y);
        return FTE_ERR_UNSUPPORTED;
    }
    *o = bestp;
    o->form = best_form;
    return FTE_OK;
}

int fte_choose_params_ex(int kind, int64_t nsrc, int64_t ntar, double Q, double Lx, double Ly, const fte_options* opt,
                         fte_params* out) {
    if (opt && opt->form == FTE_FORM_MIXED) return choose_params_tuned(kind, nsrc, ntar, Q, Lx, Ly, opt, out);
    return choose_params_q(kind, nsrc, ntar, Q, Lx, Ly, opt, out);
}

extern "C" int fte_choose_params(int kind, int64_t nsrc, int64_t ntar, const double* f1, const double* f2, double Lx,
                                 double Ly, const fte_options* opt, fte_params* out) {
    if (!out || (nsrc > 0 && (!f1 || !f2))) {
        fte_set_error("fte_choose_params: null argument");
        return FTE_ERR_INVALID;
    }
    if (!(Lx > 0) || !(Ly > 0) || !std::isfinite(Lx) || !std::isfinite(Ly)) {
        fte_set_error("fte_choose_params: box lengths must be positive and finite");
        return FTE_ERR_INVALID;
    }
    double Q = 0;
    const double* w = opt ? opt->weights : nullptr;
    for (int64_t j = 0; j < nsrc; j++) {
        double a = f1[j] * (w ? w[j] : 1.0);
        Q += a * a;
    }
    for (int64_t j = 0; j < nsrc; j++) {
        double a = f2[j] * (w ? w[j] : 1.0);
        Q += a * a;
    }
    if (opt && opt->form == FTE_FORM_MIXED) return choose_params_tuned(kind, nsrc, ntar, Q + 1, Lx, Ly, opt, out);
    return choose_params_q(kind, nsrc, ntar, Q + 1, Lx, Ly, opt, out);
}

// ---------------------------------------------------------------------------
// small device kernels of the drivers
// ---------------------------------------------------------------------------
namespace {

__global__ void k_wrap_pack(const double* __restrict__ x, const double* __restrict__ y, int64_t n, double Lx,
                            double Ly, double* __restrict__ p) {
    const double rLx = __drcp_rn(Lx), rLy = __drcp_rn(Ly);
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
        p[2 * i] = fte_wrap_coord(x[i], Lx, rLx);
        p[2 * i + 1] = fte_wrap_coord(y[i], Ly, rLy);
    }
}

__global__ void k_pack(const double* __restrict__ a, const double* __restrict__ b, int64_t n, double* __restrict__ p) {
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
        p[2 * i] = a[i];
        p[2 * i + 1] = b[i];
    }
}

// block sums of up to three values added to acc[0 .. count-1] (one atomic
// each per block)
__device__ __forceinline__ void block_acc3(double q, double zx, double zy, double* __restrict__ acc, int count) {
    for (int o = 16; o > 0; o >>= 1) {
        q += __shfl_down_sync(0xffffffffu, q, o);
        zx += __shfl_down_sync(0xffffffffu, zx, o);
        zy += __shfl_down_sync(0xffffffffu, zy, o);
    }
    __shared__ double sq[32], sx[32], sy[32];
    int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    if (lane == 0) {
        sq[warp] = q;
        sx[warp] = zx;
        sy[warp] = zy;
    }
    __syncthreads();
    if (warp == 0) {
        int nw = blockDim.x >> 5;
        q = lane < nw ? sq[lane] : 0;
        zx = lane < nw ? sx[lane] : 0;
        zy = lane < nw ? sy[lane] : 0;
        for (int o = 16; o > 0; o >>= 1) {
            q += __shfl_down_sync(0xffffffffu, q, o);
            zx += __shfl_down_sync(0xffffffffu, zx, o);
            zy += __shfl_down_sync(0xffffffffu, zy, o);
        }
        if (lane == 0) {
            atomicAdd(&acc[0], q);
            if (count > 1) atomicAdd(&acc[1], zx);
            if (count > 2) atomicAdd(&acc[2], zy);
        }
    }
}

// acc[0] += sum (w f1)^2 + (w f2)^2, the estimates' Q, from the caller's
// (staged) density and weight arrays: it needs no packing, so the host can
// read it back while the wrapping kernels run
__global__ void k_reduce_q(const double* __restrict__ f1, const double* __restrict__ f2,
                           const double* __restrict__ wts, int64_t n, double* __restrict__ acc) {
    double q = 0;
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
        const double w = wts ? wts[i] : 1.0;
        const double a = f1[i] * w, b = f2[i] * w;
        q += a * a + b * b;
    }
    block_acc3(q, 0.0, 0.0, acc, 1);
}

// acc[1..2] += sum (w f . n) (xs, ys) over the wrapped sources: the
// stresslet's zero mode
__global__ void k_reduce_zero(const double* __restrict__ p, const double* __restrict__ f,
                              const double* __restrict__ nrm, const double* __restrict__ wts, int64_t n,
                              double* __restrict__ acc) {
    double zx = 0, zy = 0;
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
        const double w = wts ? wts[i] : 1.0;
        const double fn = f[2 * i] * w * nrm[2 * i] + f[2 * i + 1] * w * nrm[2 * i + 1];
        zx += fn * p[2 * i];
        zy += fn * p[2 * i + 1];
    }
    block_acc3(zx, zy, 0.0, acc + 1, 2);
}

// u = ur + uk (+ zero mode); optional interleaved copies of ur and uk (with the zero mode in uk)
__global__ void k_combine(const double2* __restrict__ ur, const double2* __restrict__ uk, int64_t n,
                          const double* __restrict__ zero, double inv_area, double* __restrict__ u1,
                          double* __restrict__ u2, double* __restrict__ ur_out, double* __restrict__ uk_out) {
    double zx = zero ? zero[1] * inv_area : 0.0, zy = zero ? zero[2] * inv_area : 0.0;
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
        double2 r = ur[i], k = uk[i];
        k.x += zx;
        k.y += zy;
        u1[i] = r.x + k.x;
        u2[i] = r.y + k.y;
        if (ur_out) {
            ur_out[2 * i] = r.x;
            ur_out[2 * i + 1] = r.y;
        }
        if (uk_out) {
            uk_out[2 * i] = k.x;
            uk_out[2 * i + 1] = k.y;
        }
    }
}

int grid1d(fte_context* c, int64_t n, int threads = 256) {
    int64_t b = (n + threads - 1) / threads;
    int64_t mx = (int64_t)c->num_sms * 8;
    if (b > mx) b = mx;
    if (b < 1) b = 1;
    return (int)b;
}

// ---- validation -------------------------------------------------------------
int check_box(double Lx, double Ly) {
    if (!(Lx > 0) || !(Ly > 0) || !std::isfinite(Lx) || !std::isfinite(Ly)) {
        fte_set_error("box lengths must be positive and finite (Lx=%g, Ly=%g)", Lx, Ly);
        return FTE_ERR_INVALID;
    }
    return FTE_OK;
}

int check_counts(int64_t nsrc, int64_t ntar) {
    if (nsrc < 0 || ntar < 0 || nsrc > 2000000000LL || ntar > 2000000000LL) {
        fte_set_error("point counts out of range (nsrc=%lld, ntar=%lld)", (long long)nsrc, (long long)ntar);
        return FTE_ERR_INVALID;
    }
    return FTE_OK;
}

int check_real_params(double xi, int nsx, int nsy) {
    if (!(xi > 0) || !std::isfinite(xi)) {
        fte_set_error("xi must be positive and finite (xi=%g)", xi);
        return FTE_ERR_INVALID;
    }
    if (nsx < 1 || nsy < 1 || (int64_t)nsx * nsy > 100000000LL) {
        fte_set_error("cell counts out of range (nside_x=%d, nside_y=%d)", nsx, nsy);
        return FTE_ERR_INVALID;
    }
    return FTE_OK;
}

// equal_steps: the reference's requirement Lx / Mx = Ly / My (gateways and
// the drivers' form); the mixed form's tuned choice may give each axis its own
// step
int check_kspace_params(double xi, double eta, int Mx, int My, double Lx, double Ly, double w, int P,
                        bool equal_steps = true) {
    if (!(xi > 0) || !std::isfinite(xi) || !(eta > 0) || !std::isfinite(eta) || !std::isfinite(w)) {
        fte_set_error("xi, eta must be positive and w finite (xi=%g, eta=%g, w=%g)", xi, eta, w);
        return FTE_ERR_INVALID;
    }
    if (P < 2 || P % 2 != 0 || P > 64) {
        fte_set_error("window support P must be even and in [2, 64] (P=%d)", P);
        return FTE_ERR_INVALID;
    }
    if (Mx < 2 || My < 2 || Mx % 2 || My % 2) {
        fte_set_error("grid sizes must be even and >= 2 (Mx=%d, My=%d)", Mx, My);
        return FTE_ERR_INVALID;
    }
    // P + 1 > M is allowed: the window then wraps around the periodic grid
    // more than once, as it does in the reference.
    if ((double)Mx * (double)My > 2147483648.0) {
        // e.g. the drivers' grid (A M, B M) of a box whose aspect ratio has
        // large rat() terms: the reference cannot hold it either
        fte_set_error("grid of %d x %d nodes exceeds 2^31 nodes (a box whose aspect ratio Lx/Ly is no small "
                      "rational needs the mixed form's tuned choice)", Mx, My);
        return FTE_ERR_UNSUPPORTED;
    }
    double hx = Lx / Mx, hy = Ly / My;
    if (equal_steps && std::fabs(hx - hy) > 1e-12 * std::fmax(hx, hy)) {
        fte_set_error("grid spacing must be equal in x and y (Lx/Mx=%.17g, Ly/My=%.17g)", hx, hy);
        return FTE_ERR_INVALID;
    }
    return FTE_OK;
}

// Stage host arrays in device workspace when the call uses host pointers.
struct Stager {
    fte_context* c;
    WsCarver* wc;
    bool host;
    int put(const double* src, size_t count, const double** dst) {
        if (!host || !src) {
            *dst = src;
            return FTE_OK;
        }
        double* d = wc->take<double>(count);
        if (count) FTE_CUDA_TRY(cudaMemcpyAsync(d, src, count * sizeof(double), cudaMemcpyHostToDevice, c->stream));
        *dst = d;
        return FTE_OK;
    }
};

int finish_output(fte_context* c, bool host, double* user, const double* dev, size_t count) {
    if (host && user && count)
        FTE_CUDA_TRY(cudaMemcpyAsync(user, dev, count * sizeof(double), cudaMemcpyDeviceToHost, c->stream));
    return FTE_OK;
}

}  // namespace

// ---------------------------------------------------------------------------
// gateway-level entries
// ---------------------------------------------------------------------------
static int real_entry(fte_context* c, int kind, const double* psrc, int64_t nsrc, const double* ptar, int64_t ntar,
                      const double* f, const double* nrm, double xi, int nsx, int nsy, double Lx, double Ly,
                      double* ur, unsigned flags) {
    if (!c) {
        fte_set_error("null context");
        return FTE_ERR_INVALID;
    }
    FTE_TRY(check_counts(nsrc, ntar));
    FTE_TRY(check_box(Lx, Ly));
    FTE_TRY(check_real_params(xi, nsx, nsy));
    if ((nsrc > 0 && (!psrc || !f || (kind == FTE_KIND_DLP && !nrm))) || (ntar > 0 && (!ptar || !ur))) {
        fte_set_error("null array argument");
        return FTE_ERR_INVALID;
    }
    FTE_CUDA_TRY(cudaSetDevice(c->device));
    const bool host = !(flags & FTE_DEVICE_POINTERS);
    int nb = nsx * nsy;
    size_t need = fte_cells_ws(nsrc, ntar, nb) + ws_bytes(2 * (ntar + 1), sizeof(double));
    if (host) need += ws_bytes(2 * (nsrc + 1), 8) * 3 + ws_bytes(2 * (ntar + 1), 8);
    FTE_TRY(fte_ws_reserve(c, need));
    WsCarver wc{c->ws, 0, c->ws_size};
    Stager st{c, &wc, host};
    const double *dps, *dpt, *df, *dn;
    FTE_TRY(st.put(psrc, 2 * (size_t)nsrc, &dps));
    FTE_TRY(st.put(ptar, 2 * (size_t)ntar, &dpt));
    FTE_TRY(st.put(f, 2 * (size_t)nsrc, &df));
    FTE_TRY(st.put(kind == FTE_KIND_DLP ? nrm : nullptr, 2 * (size_t)nsrc, &dn));
    double2* dur = host ? wc.take<double2>(ntar + 1) : reinterpret_cast<double2*>(ur);
    FTE_WS_CHECK(wc);
    FiniteSet fin;
    fin.add(dps, 2 * nsrc);
    fin.add(dpt, 2 * ntar);
    fin.add(df, 2 * nsrc);
    fin.add(dn, 2 * nsrc);
    FTE_TRY(fte_check_finite(c, fin, kind == FTE_KIND_SLP ? "fte_slp_real" : "fte_dlp_real"));
    if (ntar > 0) {
        CellList cl;
        FTE_TRY(fte_cells_build(c, wc, kind, dps, nsrc, dpt, ntar, df, dn, nullptr, nsx, nsy, Lx, Ly, &cl));
        FTE_TRY(fte_near_launch(c, kind, cl, xi, Lx, Ly, dur));
        FTE_TRY(finish_output(c, host, ur, reinterpret_cast<const double*>(dur), 2 * (size_t)ntar));
    }
    FTE_CUDA_TRY(cudaStreamSynchronize(c->stream));
    return FTE_OK;
}

extern "C" int fte_slp_real(fte_context* c, const double* psrc, int64_t nsrc, const double* ptar, int64_t ntar,
                            const double* f, double xi, int nside_x, int nside_y, double Lx, double Ly, double* ur,
                            unsigned flags) {
    return real_entry(c, FTE_KIND_SLP, psrc, nsrc, ptar, ntar, f, nullptr, xi, nside_x, nside_y, Lx, Ly, ur, flags);
}

extern "C" int fte_dlp_real(fte_context* c, const double* psrc, int64_t nsrc, const double* ptar, int64_t ntar,
                            const double* f, const double* n, double xi, int nside_x, int nside_y, double Lx,
                            double Ly, double* ur, unsigned flags) {
    return real_entry(c, FTE_KIND_DLP, psrc, nsrc, ptar, ntar, f, n, xi, nside_x, nside_y, Lx, Ly, ur, flags);
}

static int kspace_entry(fte_context* c, int kind, const double* psrc, int64_t nsrc, const double* ptar, int64_t ntar,
                        double xi, double eta, const double* f, const double* nrm, int Mx, int My, double Lx,
                        double Ly, double w, int P, double* uk, unsigned flags) {
    if (!c) {
        fte_set_error("null context");
        return FTE_ERR_INVALID;
    }
    FTE_TRY(check_counts(nsrc, ntar));
    FTE_TRY(check_box(Lx, Ly));
    FTE_TRY(check_kspace_params(xi, eta, Mx, My, Lx, Ly, w, P));
    if ((nsrc > 0 && (!psrc || !f || (kind == FTE_KIND_DLP && !nrm))) || (ntar > 0 && (!ptar || !uk))) {
        fte_set_error("null array argument");
        return FTE_ERR_INVALID;
    }
    FTE_CUDA_TRY(cudaSetDevice(c->device));
    const bool host = !(flags & FTE_DEVICE_POINTERS);
    size_t need = fte_kspace_ws(kind, FTE_FORM_PLAIN, Mx, My, nsrc, ntar) + ws_bytes(2 * (ntar + 1), 8);
    if (host) need += ws_bytes(2 * (nsrc + 1), 8) * 3 + ws_bytes(2 * (ntar + 1), 8);
    FTE_TRY(fte_ws_reserve(c, need));
    WsCarver wc{c->ws, 0, c->ws_size};
    Stager st{c, &wc, host};
    const double *dps, *dpt, *df, *dn;
    FTE_TRY(st.put(psrc, 2 * (size_t)nsrc, &dps));
    FTE_TRY(st.put(ptar, 2 * (size_t)ntar, &dpt));
    FTE_TRY(st.put(f, 2 * (size_t)nsrc, &df));
    FTE_TRY(st.put(kind == FTE_KIND_DLP ? nrm : nullptr, 2 * (size_t)nsrc, &dn));
    double2* duk = host ? wc.take<double2>(ntar + 1) : reinterpret_cast<double2*>(uk);
    FTE_WS_CHECK(wc);
    FiniteSet fin;
    fin.add(dps, 2 * nsrc);
    fin.add(dpt, 2 * ntar);
    fin.add(df, 2 * nsrc);
    fin.add(dn, 2 * nsrc);
    FTE_TRY(fte_check_finite(c, fin, kind == FTE_KIND_SLP ? "fte_slp_kspace" : "fte_dlp_kspace"));
    KspaceArgs a;
    a.kind = kind;
    a.form = FTE_FORM_PLAIN;
    a.nsrc = nsrc;
    a.ntar = ntar;
    a.psrc = dps;
    a.ptar = dpt;
    a.f = df;
    a.nrm = dn;
    a.wts = nullptr;
    a.xi = xi;
    a.eta = eta;
    a.w = w;
    a.Lx = Lx;
    a.Ly = Ly;
    a.Mx = Mx;
    a.My = My;
    a.P = P;
    a.uk = duk;
    FTE_TRY(fte_kspace_run(c, wc, a, nullptr));
    FTE_TRY(finish_output(c, host, uk, reinterpret_cast<const double*>(duk), 2 * (size_t)ntar));
    FTE_CUDA_TRY(cudaStreamSynchronize(c->stream));
    return FTE_OK;
}

// ---------------------------------------------------------------------------
// other quantities, gateway level
// ---------------------------------------------------------------------------
extern "C" int fte_q_ncomp(int q) {
    switch (q) {
        case FTE_Q_VELOCITY: return 2;
        case FTE_Q_PRESSURE: return 1;
        case FTE_Q_PRESSURE_GRAD: return 2;
        case FTE_Q_GRADIENT: return 4;
        case FTE_Q_STRESS: return 4;
        case FTE_Q_VORTICITY: return 1;
        default: return 0;
    }
}

static int check_q(int kind, int q) {
    if (kind != FTE_KIND_SLP && kind != FTE_KIND_DLP) {
        fte_set_error("unknown kind %d", kind);
        return FTE_ERR_INVALID;
    }
    if (q < FTE_Q_PRESSURE || q > FTE_Q_VORTICITY) {
        fte_set_error("quantity %d is not one of FTE_Q_PRESSURE .. FTE_Q_VORTICITY", q);
        return FTE_ERR_INVALID;
    }
    return FTE_OK;
}

extern "C" int fte_q_real(fte_context* c, int kind, int q, const double* psrc, int64_t nsrc, const double* ptar,
                          int64_t ntar, const double* f, const double* n, double xi, int nsx, int nsy, double Lx,
                          double Ly, double* out, unsigned flags) {
    if (!c) {
        fte_set_error("null context");
        return FTE_ERR_INVALID;
    }
    FTE_TRY(check_q(kind, q));
    FTE_TRY(check_counts(nsrc, ntar));
    FTE_TRY(check_box(Lx, Ly));
    FTE_TRY(check_real_params(xi, nsx, nsy));
    if ((nsrc > 0 && (!psrc || !f || (kind == FTE_KIND_DLP && !n))) || (ntar > 0 && (!ptar || !out))) {
        fte_set_error("null array argument");
        return FTE_ERR_INVALID;
    }
    FTE_CUDA_TRY(cudaSetDevice(c->device));
    const bool host = !(flags & FTE_DEVICE_POINTERS);
    const int nc = fte_q_ncomp(q);
    size_t need = fte_cells_ws(nsrc, ntar, nsx * nsy) + ws_bytes((size_t)nc * (ntar + 1), 8);
    if (host) need += ws_bytes(2 * (nsrc + 1), 8) * 3 + ws_bytes(2 * (ntar + 1), 8);
    FTE_TRY(fte_ws_reserve(c, need));
    WsCarver wc{c->ws, 0, c->ws_size};
    Stager st{c, &wc, host};
    const double *dps, *dpt, *df, *dn;
    FTE_TRY(st.put(psrc, 2 * (size_t)nsrc, &dps));
    FTE_TRY(st.put(ptar, 2 * (size_t)ntar, &dpt));
    FTE_TRY(st.put(f, 2 * (size_t)nsrc, &df));
    FTE_TRY(st.put(kind == FTE_KIND_DLP ? n : nullptr, 2 * (size_t)nsrc, &dn));
    double* dout = host ? wc.take<double>((size_t)nc * (ntar + 1)) : out;
    FTE_WS_CHECK(wc);
    FiniteSet fin;
    fin.add(dps, 2 * nsrc);
    fin.add(dpt, 2 * ntar);
    fin.add(df, 2 * nsrc);
    fin.add(dn, 2 * nsrc);
    FTE_TRY(fte_check_finite(c, fin, "fte_q_real"));
    if (ntar > 0) {
        CellList cl;
        FTE_TRY(fte_cells_build(c, wc, kind, dps, nsrc, dpt, ntar, df, dn, nullptr, nsx, nsy, Lx, Ly, &cl));
        FTE_TRY(fte_q_near_launch(c, kind, q, cl, df, dn, xi, Lx, Ly, dout));
        FTE_TRY(finish_output(c, host, out, dout, (size_t)nc * ntar));
    }
    FTE_CUDA_TRY(cudaStreamSynchronize(c->stream));
    return FTE_OK;
}

extern "C" int fte_q_kspace(fte_context* c, int kind, int q, const double* psrc, int64_t nsrc, const double* ptar,
                            int64_t ntar, const double* f, const double* n, double xi, double eta, int Mx, int My,
                            double Lx, double Ly, double w, int P, double* out, unsigned flags) {
    if (!c) {
        fte_set_error("null context");
        return FTE_ERR_INVALID;
    }
    FTE_TRY(check_q(kind, q));
    FTE_TRY(check_counts(nsrc, ntar));
    FTE_TRY(check_box(Lx, Ly));
    FTE_TRY(check_kspace_params(xi, eta, Mx, My, Lx, Ly, w, P));
    if ((nsrc > 0 && (!psrc || !f || (kind == FTE_KIND_DLP && !n))) || (ntar > 0 && (!ptar || !out))) {
        fte_set_error("null array argument");
        return FTE_ERR_INVALID;
    }
    FTE_CUDA_TRY(cudaSetDevice(c->device));
    const bool host = !(flags & FTE_DEVICE_POINTERS);
    const int nc = fte_q_ncomp(q);
    size_t need = fte_q_kspace_ws(Mx, My, nsrc, ntar) + ws_bytes((size_t)nc * (ntar + 1), 8);
    if (host) need += ws_bytes(2 * (nsrc + 1), 8) * 3 + ws_bytes(2 * (ntar + 1), 8);
    FTE_TRY(fte_ws_reserve(c, need));
    WsCarver wc{c->ws, 0, c->ws_size};
    Stager st{c, &wc, host};
    const double *dps, *dpt, *df, *dn;
    FTE_TRY(st.put(psrc, 2 * (size_t)nsrc, &dps));
    FTE_TRY(st.put(ptar, 2 * (size_t)ntar, &dpt));
    FTE_TRY(st.put(f, 2 * (size_t)nsrc, &df));
    FTE_TRY(st.put(kind == FTE_KIND_DLP ? n : nullptr, 2 * (size_t)nsrc, &dn));
    double* dout = host ? wc.take<double>((size_t)nc * (ntar + 1)) : out;
    FTE_WS_CHECK(wc);
    FiniteSet fin;
    fin.add(dps, 2 * nsrc);
    fin.add(dpt, 2 * ntar);
    fin.add(df, 2 * nsrc);
    fin.add(dn, 2 * nsrc);
    FTE_TRY(fte_check_finite(c, fin, "fte_q_kspace"));
    KspaceArgs a;
    a.kind = kind;
    a.form = FTE_FORM_PLAIN;
    a.nsrc = nsrc;
    a.ntar = ntar;
    a.psrc = dps;
    a.ptar = dpt;
    a.f = df;
    a.nrm = dn;
    a.wts = nullptr;
    a.xi = xi;
    a.eta = eta;
    a.w = w;
    a.Lx = Lx;
    a.Ly = Ly;
    a.Mx = Mx;
    a.My = My;
    a.P = P;
    a.uk = nullptr;
    FTE_TRY(fte_q_kspace_run(c, wc, q, a, dout));
    FTE_TRY(finish_output(c, host, out, dout, (size_t)nc * ntar));
    FTE_CUDA_TRY(cudaStreamSynchronize(c->stream));
    return FTE_OK;
}

extern "C" int fte_slp_kspace(fte_context* c, const double* psrc, int64_t nsrc, const double* ptar, int64_t ntar,
                              double xi, double eta, const double* f, int Mx, int My, double Lx, double Ly, double w,
                              int P, double* uk, unsigned flags) {
    return kspace_entry(c, FTE_KIND_SLP, psrc, nsrc, ptar, ntar, xi, eta, f, nullptr, Mx, My, Lx, Ly, w, P, uk, flags);
}

extern "C" int fte_dlp_kspace(fte_context* c, const double* psrc, int64_t nsrc, const double* ptar, int64_t ntar,
                              double xi, double eta, const double* f, const double* n, int Mx, int My, double Lx,
                              double Ly, double w, int P, double* uk, unsigned flags) {
    return kspace_entry(c, FTE_KIND_DLP, psrc, nsrc, ptar, ntar, xi, eta, f, n, Mx, My, Lx, Ly, w, P, uk, flags);
}

// ---------------------------------------------------------------------------
// driver-level entries
// ---------------------------------------------------------------------------
static int ewald_entry(fte_context* c, int kind, const double* xsrc, const double* ysrc, int64_t nsrc,
                       const double* xtar, const double* ytar, int64_t ntar, const double* n1, const double* n2,
                       const double* f1, const double* f2, double Lx, double Ly, const fte_options* opt, double* u1,
                       double* u2, double* ur, double* uk, fte_info* info, unsigned flags) {
    if (!c) {
        fte_set_error("null context");
        return FTE_ERR_INVALID;
    }
    FTE_TRY(check_counts(nsrc, ntar));
    FTE_TRY(check_box(Lx, Ly));
    if ((nsrc > 0 && (!xsrc || !ysrc || !f1 || !f2 || (kind == FTE_KIND_DLP && (!n1 || !n2)))) ||
        (ntar > 0 && (!xtar || !ytar || !u1 || !u2))) {
        fte_set_error("null array argument");
        return FTE_ERR_INVALID;
    }
    fte_options defaults;
    std::memset(&defaults, 0, sizeof(defaults));
    if (!opt) opt = &defaults;
    if (opt->P != 0 && (opt->P < 2 || opt->P % 2 || opt->P > 64)) {
        fte_set_error("window support P must be even and in [2, 64] (P=%d)", opt->P);
        return FTE_ERR_INVALID;
    }
    if (opt->form != FTE_FORM_PLAIN && opt->form != FTE_FORM_MIXED) {
        fte_set_error("unknown form %d", opt->form);
        return FTE_ERR_INVALID;
    }
    FTE_CUDA_TRY(cudaSetDevice(c->device));
    const bool host = !(flags & FTE_DEVICE_POINTERS);
    long long k0 = c->kernels;
    FTE_TRY(fte_record(c, 0));

    // workspace (first pass: everything except the grids, which need the parameters)
    size_t base = 0;
    base += ws_bytes(2 * (nsrc + 1), 8) * 3 + ws_bytes(2 * (ntar + 1), 8) * 3;  // packed inputs + ur/uk
    if (host) base += ws_bytes(nsrc + 1, 8) * 7 + ws_bytes(ntar + 1, 8) * 8;
    base += 4096;
    FTE_TRY(fte_ws_reserve(c, base));
    // host inputs are staged first so that Q can be reduced on the device
    WsCarver wc{c->ws, 0, c->ws_size};
    Stager st{c, &wc, host};
    const double *dxs, *dys, *dxt, *dyt, *df1, *df2, *dn1 = nullptr, *dn2 = nullptr, *dw = nullptr;
    FTE_TRY(st.put(xsrc, nsrc, &dxs));
    FTE_TRY(st.put(ysrc, nsrc, &dys));
    FTE_TRY(st.put(xtar, ntar, &dxt));
    FTE_TRY(st.put(ytar, ntar, &dyt));
    FTE_TRY(st.put(f1, nsrc, &df1));
    FTE_TRY(st.put(f2, nsrc, &df2));
    if (kind == FTE_KIND_DLP) {
        FTE_TRY(st.put(n1, nsrc, &dn1));
        FTE_TRY(st.put(n2, nsrc, &dn2));
    }
    FTE_TRY(st.put(opt->weights, nsrc, &dw));
    double* ps = wc.take<double>(2 * (nsrc + 1));
    double* pt = wc.take<double>(2 * (ntar + 1));
    double* pf = wc.take<double>(2 * (nsrc + 1));
    double* pn = kind == FTE_KIND_DLP ? wc.take<double>(2 * (nsrc + 1)) : nullptr;
    double2* dur = wc.take<double2>(ntar + 1);
    double2* duk = wc.take<double2>(ntar + 1);
    double* acc = wc.take<double>(8);
    FTE_WS_CHECK(wc);
    FiniteSet fin;
    for (const double* a : {dxs, dys, df1, df2, dn1, dn2, dw}) fin.add(a, nsrc);
    fin.add(dxt, ntar);
    fin.add(dyt, ntar);
    // the input check and Q first: the host reads them back (event ev_q)
    // and chooses the parameters while the wrapping and packing kernels run
    FTE_TRY(fte_finite_launch(c, fin));
    FTE_CUDA_TRY(cudaMemsetAsync(acc, 0, 8 * sizeof(double), c->stream));
    if (nsrc > 0) FTE_LAUNCH(c, k_reduce_q, grid1d(c, nsrc), 256, 0, df1, df2, dw, nsrc, acc);
    FTE_CUDA_TRY(cudaMemcpyAsync(c->host_scalars, acc, sizeof(double), cudaMemcpyDeviceToHost, c->stream));
    FTE_CUDA_TRY(cudaEventRecord(c->ev_q, c->stream));
    if (nsrc > 0) {
        FTE_LAUNCH(c, k_wrap_pack, grid1d(c, nsrc), 256, 0, dxs, dys, nsrc, Lx, Ly, ps);
        FTE_LAUNCH(c, k_pack, grid1d(c, nsrc), 256, 0, df1, df2, nsrc, pf);
        if (pn) FTE_LAUNCH(c, k_pack, grid1d(c, nsrc), 256, 0, dn1, dn2, nsrc, pn);
    }
    if (ntar > 0) FTE_LAUNCH(c, k_wrap_pack, grid1d(c, ntar), 256, 0, dxt, dyt, ntar, Lx, Ly, pt);
    if (nsrc > 0 && kind == FTE_KIND_DLP)
        FTE_LAUNCH(c, k_reduce_zero, grid1d(c, nsrc), 256, 0, (const double*)ps, (const double*)pf,
                   (const double*)pn, dw, nsrc, acc);
    FTE_CUDA_TRY(cudaEventSynchronize(c->ev_q));
    FTE_TRY(fte_finite_result(c, kind == FTE_KIND_SLP ? "fte_stokes_slp_ewald_2p" : "fte_stokes_dlp_ewald_2p"));
    double Q = c->host_scalars[0] + 1.0;
    fte_params prm;
    if (opt->form == FTE_FORM_MIXED)
        FTE_TRY(choose_params_tuned(kind, nsrc, ntar, Q, Lx, Ly, opt, &prm));
    else
        FTE_TRY(choose_params_q(kind, nsrc, ntar, Q, Lx, Ly, opt, &prm));
    FTE_TRY(check_real_params(prm.xi, prm.nside_x, prm.nside_y));
    FTE_TRY(check_kspace_params(prm.xi, prm.eta, prm.Mx, prm.My, Lx, Ly, prm.w, prm.P, opt->form != FTE_FORM_MIXED));
    // second workspace: cell list, grids and outputs (the staged point data stays in the first)
    size_t need = fte_cells_ws(nsrc, ntar, prm.nside_x * prm.nside_y) +
                  fte_kspace_ws(kind, prm.form, prm.Mx, prm.My, nsrc, ntar) + ws_bytes(2 * (ntar + 1), 8) * 3 +
                  fte_near_ff_ws(kind, 1, nsrc) + 8192;
    FTE_TRY(fte_ws2_reserve(c, need));
    WsCarver wc2{c->ws2, 0, c->ws2_size};
    FTE_TRY(fte_record(c, 1));
    if (ntar > 0) {
        CellList cl;
        FTE_TRY(fte_cells_build(c, wc2, kind, ps, nsrc, pt, ntar, pf, pn, dw, prm.nside_x, prm.nside_y, Lx, Ly, &cl));
        if (opt->form == FTE_FORM_MIXED) cl.cutoffsq = fte_tuned_cutoffsq(prm, Lx, Ly);
        FTE_TRY(fte_record(c, 6));
        // the mixed form evaluates the pairs whose terms are far below the
        // tolerance in FP32 and the other pairs with x >= 1 in float-float
        double x32;
        bool ffn;
        FTE_TRY(fte_near_classes(opt, prm.tol, &x32, &ffn));
        void* ffmem = nullptr;
        if (ffn) {
            ffmem = wc2.take<char>(fte_near_ff_ws(kind, 1, nsrc));
            FTE_WS_CHECK(wc2);
        }
        FTE_TRY(fte_near_launch(c, kind, cl, prm.xi, Lx, Ly, dur, x32, ffn, ffmem));
        FTE_TRY(fte_record(c, 7));
        KspaceArgs a;
        a.kind = kind;
        a.form = prm.form;
        a.nsrc = nsrc;
        a.ntar = ntar;
        a.psrc = ps;
        a.ptar = pt;
        a.f = pf;
        a.nrm = pn;
        a.wts = dw;
        a.xi = prm.xi;
        a.eta = prm.eta;
        a.w = prm.w;
        a.Lx = Lx;
        a.Ly = Ly;
        a.Mx = prm.Mx;
        a.My = prm.My;
        a.P = prm.P;
        a.uk = duk;
        FTE_TRY(fte_kspace_run(c, wc2, a, info));
        double* ou1 = host ? wc2.take<double>(ntar + 1) : u1;
        double* ou2 = host ? wc2.take<double>(ntar + 1) : u2;
        double* our = (ur && host) ? wc2.take<double>(2 * (ntar + 1)) : ur;
        double* ouk = (uk && host) ? wc2.take<double>(2 * (ntar + 1)) : uk;
        FTE_WS_CHECK(wc2);
        FTE_LAUNCH(c, k_combine, grid1d(c, ntar), 256, 0, (const double2*)dur, (const double2*)duk, ntar,
                   kind == FTE_KIND_DLP ? (const double*)acc : nullptr, 1.0 / (Lx * Ly), ou1, ou2, our, ouk);
        FTE_TRY(fte_record(c, 5));
        if (host) {
            FTE_TRY(finish_output(c, true, u1, ou1, ntar));
            FTE_TRY(finish_output(c, true, u2, ou2, ntar));
            FTE_TRY(finish_output(c, true, ur, our, 2 * (size_t)ntar));
            FTE_TRY(finish_output(c, true, uk, ouk, 2 * (size_t)ntar));
        }
    }
    FTE_CUDA_TRY(cudaStreamSynchronize(c->stream));
    if (info) {
        std::memset(info, 0, sizeof(*info));
        info->params = prm;
        info->kernels_launched = (int)(c->kernels - k0);
        if (c->timing && ntar > 0) {
            info->ms_total = fte_elapsed(c, 0, 5);
            info->ms_cells = fte_elapsed(c, 1, 6);
            info->ms_near = fte_elapsed(c, 6, 7);
            info->ms_spread = fte_elapsed(c, 2, 3);
            info->ms_fft = fte_elapsed(c, 3, 4);
            info->ms_gather = fte_elapsed(c, 4, 5);
        }
    }
    return FTE_OK;
}

// ---------------------------------------------------------------------------
// other quantities, driver level: StokesSLP_<q>_ewald_2p / StokesDLP_<q>_ewald_2p
// (PeriodicEwald/src/matlab/), q = pressure, pressure_grad, gradient, stress,
// vorticity.  As the MATLAB drivers: wrap the points, choose the parameters
// (the velocity drivers' estimates; the stresslet vorticity driver uses the
// Stokeslet's), call the gateways, then per quantity
//   SLP pressure:  p  = pr + pk,  pk = k-space - sum(f1 x + f2 y) / (2 Lx Ly)
//   DLP pressure:  p  = pr + pk + pself,  pk = k-space - sum(n.f) / (2 Lx Ly),
//                  pself = xi^2 (f.n) / (2 pi) of a source at the target
//   SLP pressure gradient:  p = -(pr + pk + pself),  pself = xi^2 f / (2 pi)
//   DLP pressure gradient:  p = -2 (pr + pk)
//   velocity gradient (b):  u_1 = T1 b1 + T3 b2,  u_2 = T2 b1 + T4 b2 for the
//                  real and k parts; DLP adds uself = xi^2 (q Re(b n*) +
//                  n Re(q b*) + b Re(q n*)) / (2 pi) (complex q = f1 + i f2 ...)
//   SLP stress (b): as the gradient, plus sum(f1 x + f2 y) / (2 Lx Ly) on both
//                  components
//   DLP stress (b): real part contracted (T1 b1 + T2 b2, T3 b1 + T4 b2), k part
//                  as the gradient plus sum(n.f) / (2 Lx Ly); self term
//                  -pself on the first component (pself = xi^2 b Re(q n*) /
//                  (2 pi), complex in the driver: its real part is kept) and
//                  2 uself
//   SLP vorticity:  omega = omegar + omegak - sum(f1 y - f2 x) / (2 Lx Ly)
//   DLP vorticity:  omega = omegar + omegak
// Self terms: the drivers take the sources that coincide with some target
// (before wrapping, exact equality) and add their terms elementwise to the
// targets (k-th such source to the k-th target), or to every target when
// there is exactly one; other counts do not fit the drivers' vector sums and
// are rejected.
// ---------------------------------------------------------------------------
namespace {
// acc[0] = sum f1^2 + f2^2, acc[1] = sum f1 x + f2 y, acc[2] = sum n.f, acc[3] = sum f1 y - f2 x
__global__ void k_q_sums(const double* __restrict__ p, const double* __restrict__ f, const double* __restrict__ nrm,
                         int64_t n, double* __restrict__ acc) {
    double a[4] = {0, 0, 0, 0};
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
        const double f1 = f[2 * i], f2 = f[2 * i + 1], x = p[2 * i], y = p[2 * i + 1];
        a[0] += f1 * f1 + f2 * f2;
        a[1] += f1 * x + f2 * y;
        if (nrm) a[2] += nrm[2 * i] * f1 + nrm[2 * i + 1] * f2;
        a[3] += f1 * y - f2 * x;
    }
#pragma unroll
    for (int c = 0; c < 4; c++) {
        double v = a[c];
        for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
        if ((threadIdx.x & 31) == 0) atomicAdd(&acc[c], v);
    }
}

__global__ void k_q_combine(int kind, int q, int64_t nt, const double* __restrict__ R, const double* __restrict__ K,
                            const double* __restrict__ b1, const double* __restrict__ b2, const int* __restrict__ eqs,
                            const double* __restrict__ f, const double* __restrict__ nrm, double xi,
                            const double* __restrict__ sums, double area2, double* __restrict__ out,
                            double* __restrict__ outr, double* __restrict__ outk) {
    const double inv2pi = 1.0 / (2 * FTE_PI);
    for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < nt; t += (int64_t)gridDim.x * blockDim.x) {
        const int s = eqs ? eqs[t] : -1;
        double q1 = 0, q2 = 0, m1 = 0, m2 = 0;
        if (s >= 0) {
            q1 = f[2 * s];
            q2 = f[2 * s + 1];
            if (nrm) {
                m1 = nrm[2 * s];
                m2 = nrm[2 * s + 1];
            }
        }
        if (q == FTE_Q_PRESSURE) {
            const double r = R[t];
            double k = K[t];
            double self = 0;
            if (kind == FTE_KIND_SLP) {
                k = k + -sums[1] / area2;
            } else {
                k = k + -(sums[2] / area2);
                if (s >= 0) self = xi * xi * (q1 * m1 + q2 * m2) * inv2pi;
            }
            out[t] = r + k + self;
            if (outr) outr[t] = r;
            if (outk) outk[t] = k;
        } else if (q == FTE_Q_PRESSURE_GRAD) {
            for (int c = 0; c < 2; c++) {
                const double r = R[2 * t + c], k = K[2 * t + c];
                double v;
                if (kind == FTE_KIND_SLP) {
                    const double self = s >= 0 ? xi * xi * (c ? q2 : q1) * inv2pi : 0.0;
                    v = -(r + k + self);
                } else {
                    v = -2 * (r + k);
                }
                out[2 * t + c] = v;
                if (outr) outr[2 * t + c] = r;
                if (outk) outk[2 * t + c] = k;
            }
        } else if (q == FTE_Q_GRADIENT || q == FTE_Q_STRESS) {
            const double B1 = b1[t], B2 = b2[t];
            const double* r4 = R + 4 * t;
            const double* k4 = K + 4 * t;
            double r_1, r_2;
            if (kind == FTE_KIND_DLP && q == FTE_Q_STRESS) {
                r_1 = r4[0] * B1 + r4[1] * B2;
                r_2 = r4[2] * B1 + r4[3] * B2;
            } else {
                r_1 = r4[0] * B1 + r4[2] * B2;
                r_2 = r4[1] * B1 + r4[3] * B2;
            }
            double k_1 = k4[0] * B1 + k4[2] * B2, k_2 = k4[1] * B1 + k4[3] * B2;
            double u_1 = r_1 + k_1, u_2 = r_2 + k_2;
            if (q == FTE_Q_STRESS) {
                if (kind == FTE_KIND_SLP) {
                    const double z = sums[1] / area2;
                    u_1 += z;
                    u_2 += z;
                } else {
                    const double z = sums[2] / area2;
                    k_1 += z;
                    k_2 += z;
                    u_1 = r_1 + k_1;
                    u_2 = r_2 + k_2;
                }
            }
            if (kind == FTE_KIND_DLP && s >= 0) {
                // complex q = f1 + i f2, n = n1 + i n2, b = b1 + i b2
                const double bn = B1 * m1 + B2 * m2;  // Re(b conj n)
                const double qb = q1 * B1 + q2 * B2;  // Re(q conj b)
                const double qn = q1 * m1 + q2 * m2;  // Re(q conj n)
                const double s1 = xi * xi * (q1 * bn + m1 * qb + B1 * qn) * inv2pi;
                const double s2 = xi * xi * (q2 * bn + m2 * qb + B2 * qn) * inv2pi;
                if (q == FTE_Q_GRADIENT) {
                    u_1 += s1;
                    u_2 += s2;
                } else {
                    const double pself_re = xi * xi * B1 * qn * inv2pi;
                    u_1 += -pself_re + 2 * s1;
                    u_2 += 2 * s2;
                }
            }
            out[2 * t] = u_1;
            out[2 * t + 1] = u_2;
            if (outr) {
                outr[2 * t] = r_1;
                outr[2 * t + 1] = r_2;
            }
            if (outk) {
                outk[2 * t] = k_1;
                outk[2 * t + 1] = k_2;
            }
        } else {  // vorticity
            const double r = R[t], k = K[t];
            double v = r + k;
            if (kind == FTE_KIND_SLP) v = v - sums[3] / area2;
            out[t] = v;
            if (outr) outr[t] = r;
            if (outk) outk[t] = k;
        }
    }
}
}  // namespace

extern "C" int fte_stokes_q_ewald_2p(fte_context* c, int kind, int q, const double* xsrc, const double* ysrc,
                                     int64_t nsrc, const double* xtar, const double* ytar, int64_t ntar,
                                     const double* n1, const double* n2, const double* f1, const double* f2,
                                     const double* b1, const double* b2, double Lx, double Ly,
                                     const fte_options* opt, double* out, double* out_real, double* out_k,
                                     fte_info* info, unsigned flags) {
    if (!c) {
        fte_set_error("null context");
        return FTE_ERR_INVALID;
    }
    FTE_TRY(check_q(kind, q));
    FTE_TRY(check_counts(nsrc, ntar));
    FTE_TRY(check_box(Lx, Ly));
    const bool with_b = q == FTE_Q_GRADIENT || q == FTE_Q_STRESS;
    if ((nsrc > 0 && (!xsrc || !ysrc || !f1 || !f2 || (kind == FTE_KIND_DLP && (!n1 || !n2)))) ||
        (ntar > 0 && (!xtar || !ytar || !out || (with_b && (!b1 || !b2))))) {
        fte_set_error("null array argument");
        return FTE_ERR_INVALID;
    }
    fte_options defaults;
    std::memset(&defaults, 0, sizeof(defaults));
    if (!opt) opt = &defaults;
    if (opt->P != 0 && (opt->P < 2 || opt->P % 2 || opt->P > 64)) {
        fte_set_error("window support P must be even and in [2, 64] (P=%d)", opt->P);
        return FTE_ERR_INVALID;
    }
    FTE_CUDA_TRY(cudaSetDevice(c->device));
    const bool host = !(flags & FTE_DEVICE_POINTERS);
    const long long k0 = c->kernels;
    const int nc = fte_q_ncomp(q);
    const int nd = (q == FTE_Q_PRESSURE || q == FTE_Q_VORTICITY) ? 1 : 2;  // driver outputs per target
    FTE_TRY(fte_record(c, 0));

    // sources coinciding with targets (before wrapping): the drivers' self terms
    const bool self_terms = (kind == FTE_KIND_DLP && (q == FTE_Q_PRESSURE || q == FTE_Q_GRADIENT ||
                                                      q == FTE_Q_STRESS)) ||
                            (kind == FTE_KIND_SLP && q == FTE_Q_PRESSURE_GRAD);
    std::vector<int> eqs;
    if (self_terms && nsrc > 0 && ntar > 0) {
        std::vector<double> hx(nsrc), hy(nsrc), tx(ntar), ty(ntar);
        const cudaMemcpyKind kd = host ? cudaMemcpyHostToHost : cudaMemcpyDeviceToHost;
        FTE_CUDA_TRY(cudaMemcpy(hx.data(), xsrc, nsrc * 8, kd));
        FTE_CUDA_TRY(cudaMemcpy(hy.data(), ysrc, nsrc * 8, kd));
        FTE_CUDA_TRY(cudaMemcpy(tx.data(), xtar, ntar * 8, kd));
        FTE_CUDA_TRY(cudaMemcpy(ty.data(), ytar, ntar * 8, kd));
        std::vector<std::pair<double, double>> tk(ntar);
        for (int64_t t = 0; t < ntar; t++) tk[t] = {tx[t], ty[t]};
        std::sort(tk.begin(), tk.end());
        std::vector<int> eq;
        for (int64_t s2 = 0; s2 < nsrc; s2++)
            if (std::binary_search(tk.begin(), tk.end(), std::make_pair(hx[s2], hy[s2]))) eq.push_back((int)s2);
        if (!eq.empty()) {
            if ((int64_t)eq.size() == ntar) {
                eqs = eq;
            } else if (eq.size() == 1) {
                eqs.assign(ntar, eq[0]);
            } else {
                fte_set_error("%zu sources coincide with targets but there are %lld targets: the driver's self "
                              "terms pair the k-th such source with the k-th target",
                              eq.size(), (long long)ntar);
                return FTE_ERR_UNSUPPORTED;
            }
        }
    }

    size_t base = ws_bytes(2 * (nsrc + 1), 8) * 3 + ws_bytes(2 * (ntar + 1), 8) +
                  2 * ws_bytes((size_t)nc * (ntar + 1), 8) + 3 * ws_bytes((size_t)nd * (ntar + 1), 8) +
                  ws_bytes(ntar + 1, 4) + 4096;
    if (host) base += ws_bytes(nsrc + 1, 8) * 6 + ws_bytes(ntar + 1, 8) * 4;
    FTE_TRY(fte_ws_reserve(c, base));
    WsCarver wc{c->ws, 0, c->ws_size};
    Stager st{c, &wc, host};
    const double *dxs, *dys, *dxt, *dyt, *df1, *df2, *dn1 = nullptr, *dn2 = nullptr, *db1 = nullptr, *db2 = nullptr;
    FTE_TRY(st.put(xsrc, nsrc, &dxs));
    FTE_TRY(st.put(ysrc, nsrc, &dys));
    FTE_TRY(st.put(xtar, ntar, &dxt));
    FTE_TRY(st.put(ytar, ntar, &dyt));
    FTE_TRY(st.put(f1, nsrc, &df1));
    FTE_TRY(st.put(f2, nsrc, &df2));
    if (kind == FTE_KIND_DLP) {
        FTE_TRY(st.put(n1, nsrc, &dn1));
        FTE_TRY(st.put(n2, nsrc, &dn2));
    }
    if (with_b) {
        FTE_TRY(st.put(b1, ntar, &db1));
        FTE_TRY(st.put(b2, ntar, &db2));
    }
    double* ps = wc.take<double>(2 * (nsrc + 1));
    double* pt = wc.take<double>(2 * (ntar + 1));
    double* pf = wc.take<double>(2 * (nsrc + 1));
    double* pn = kind == FTE_KIND_DLP ? wc.take<double>(2 * (nsrc + 1)) : nullptr;
    double* dR = wc.take<double>((size_t)nc * (ntar + 1));
    double* dK = wc.take<double>((size_t)nc * (ntar + 1));
    double* dout = host ? wc.take<double>((size_t)nd * (ntar + 1)) : out;
    double* dor = out_real ? (host ? wc.take<double>((size_t)nd * (ntar + 1)) : out_real) : nullptr;
    double* dok = out_k ? (host ? wc.take<double>((size_t)nd * (ntar + 1)) : out_k) : nullptr;
    int* deq = eqs.empty() ? nullptr : wc.take<int>(ntar + 1);
    double* acc = wc.take<double>(8);
    FTE_WS_CHECK(wc);
    FiniteSet fin;
    for (const double* a : {dxs, dys, df1, df2, dn1, dn2}) fin.add(a, nsrc);
    for (const double* a : {dxt, dyt, db1, db2}) fin.add(a, ntar);
    FTE_TRY(fte_finite_launch(c, fin));
    FTE_CUDA_TRY(cudaMemsetAsync(acc, 0, 8 * sizeof(double), c->stream));
    if (nsrc > 0) {
        FTE_LAUNCH(c, k_wrap_pack, grid1d(c, nsrc), 256, 0, dxs, dys, nsrc, Lx, Ly, ps);
        FTE_LAUNCH(c, k_pack, grid1d(c, nsrc), 256, 0, df1, df2, nsrc, pf);
        if (pn) FTE_LAUNCH(c, k_pack, grid1d(c, nsrc), 256, 0, dn1, dn2, nsrc, pn);
        FTE_LAUNCH(c, k_q_sums, grid1d(c, nsrc), 256, 0, (const double*)ps, (const double*)pf, (const double*)pn,
                   nsrc, acc);
    }
    if (ntar > 0) FTE_LAUNCH(c, k_wrap_pack, grid1d(c, ntar), 256, 0, dxt, dyt, ntar, Lx, Ly, pt);
    if (deq) FTE_CUDA_TRY(cudaMemcpyAsync(deq, eqs.data(), ntar * sizeof(int), cudaMemcpyHostToDevice, c->stream));
    FTE_CUDA_TRY(cudaMemcpyAsync(c->host_scalars, acc, 4 * sizeof(double), cudaMemcpyDeviceToHost, c->stream));
    FTE_CUDA_TRY(cudaStreamSynchronize(c->stream));
    FTE_TRY(fte_finite_result(c, "fte_stokes_q_ewald_2p"));
    const double Q = c->host_scalars[0] + 1.0;
    // the stresslet vorticity driver uses the Stokeslet's estimates and point count
    const int est_kind = (kind == FTE_KIND_DLP && q == FTE_Q_VORTICITY) ? FTE_KIND_SLP : kind;
    fte_params prm;
    FTE_TRY(choose_params_q(est_kind, nsrc, ntar, Q, Lx, Ly, opt, &prm));
    FTE_TRY(check_real_params(prm.xi, prm.nside_x, prm.nside_y));
    FTE_TRY(check_kspace_params(prm.xi, prm.eta, prm.Mx, prm.My, Lx, Ly, prm.w, prm.P));
    size_t need = fte_cells_ws(nsrc, ntar, prm.nside_x * prm.nside_y) + fte_q_kspace_ws(prm.Mx, prm.My, nsrc, ntar) +
                  8192;
    FTE_TRY(fte_ws2_reserve(c, need));
    if (ntar > 0) {
        WsCarver wc2{c->ws2, 0, c->ws2_size};
        CellList cl;
        FTE_TRY(fte_record(c, 1));
        FTE_TRY(fte_cells_build(c, wc2, kind, ps, nsrc, pt, ntar, pf, pn, nullptr, prm.nside_x, prm.nside_y, Lx, Ly,
                                &cl));
        FTE_TRY(fte_record(c, 6));
        FTE_TRY(fte_q_near_launch(c, kind, q, cl, pf, pn, prm.xi, Lx, Ly, dR));
        FTE_TRY(fte_record(c, 7));
        WsCarver wck{c->ws2, 0, c->ws2_size};
        KspaceArgs a;
        a.kind = kind;
        a.form = FTE_FORM_PLAIN;
        a.nsrc = nsrc;
        a.ntar = ntar;
        a.psrc = ps;
        a.ptar = pt;
        a.f = pf;
        a.nrm = pn;
        a.wts = nullptr;
        a.xi = prm.xi;
        a.eta = prm.eta;
        a.w = prm.w;
        a.Lx = Lx;
        a.Ly = Ly;
        a.Mx = prm.Mx;
        a.My = prm.My;
        a.P = prm.P;
        a.uk = nullptr;
        FTE_TRY(fte_q_kspace_run(c, wck, q, a, dK));
        FTE_TRY(fte_record(c, 5));
        // device copy of the sums for the combination
        double* dsums = acc;
        FTE_LAUNCH(c, k_q_combine, grid1d(c, ntar), 256, 0, kind, q, ntar, (const double*)dR, (const double*)dK, db1,
                   db2, (const int*)deq, (const double*)pf, (const double*)pn, prm.xi, (const double*)dsums,
                   2 * Lx * Ly, dout, dor, dok);
        FTE_TRY(finish_output(c, host, out, dout, (size_t)nd * ntar));
        if (out_real) FTE_TRY(finish_output(c, host, out_real, dor, (size_t)nd * ntar));
        if (out_k) FTE_TRY(finish_output(c, host, out_k, dok, (size_t)nd * ntar));
    }
    FTE_CUDA_TRY(cudaStreamSynchronize(c->stream));
    if (info) {
        std::memset(info, 0, sizeof(*info));
        info->params = prm;
        info->kernels_launched = (int)(c->kernels - k0);
        if (c->timing && ntar > 0) {
            info->ms_total = fte_elapsed(c, 0, 5);
            info->ms_cells = fte_elapsed(c, 1, 6);
            info->ms_near = fte_elapsed(c, 6, 7);
        }
    }
    return FTE_OK;
}

extern "C" int fte_stokes_slp_ewald_2p(fte_context* c, const double* xsrc, const double* ysrc, int64_t nsrc,
                                       const double* xtar, const double* ytar, int64_t ntar, const double* f1,
                                       const double* f2, double Lx, double Ly, const fte_options* opt, double* u1,
                                       double* u2, double* ur, double* uk, fte_info* info, unsigned flags) {
    return ewald_entry(c, FTE_KIND_SLP, xsrc, ysrc, nsrc, xtar, ytar, ntar, nullptr, nullptr, f1, f2, Lx, Ly, opt, u1,
                       u2, ur, uk, info, flags);
}

extern "C" int fte_stokes_dlp_ewald_2p(fte_context* c, const double* xsrc, const double* ysrc, int64_t nsrc,
                                       const double* xtar, const double* ytar, int64_t ntar, const double* n1,
                                       const double* n2, const double* f1, const double* f2, double Lx, double Ly,
                                       const fte_options* opt, double* u1, double* u2, double* ur, double* uk,
                                       fte_info* info, unsigned flags) {
    return ewald_entry(c, FTE_KIND_DLP, xsrc, ysrc, nsrc, xtar, ytar, ntar, n1, n2, f1, f2, Lx, Ly, opt, u1, u2, ur,
                       uk, info, flags);
}
