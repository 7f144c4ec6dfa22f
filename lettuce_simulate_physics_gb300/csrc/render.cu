// Orthographic density render of the resident bodies on the device: the reference's render_image
// (src/render.cpp:83-224, the CPU path behind PNG frames, lettuce-render and the live view) as
// CUDA kernels writing a headless RGB buffer.
//  - Projection: screen x = ax . (x, y, z), screen y = ay . (x, y, z) in FP64 from the float
//    positions (src/render.cpp:22-40 views: xy, xz, yz, "<yaw>,<pitch>").
//  - Centre: mass-weighted mean of the projected positions over the finite bodies (FP64).
//  - Extent (when 0): 1.2 x the 99th-percentile distance from the centre, found by a radix select
//    over the distances' float bits.
//  - Splat: every body's mass is shared bilinearly by the four pixels around its position. The
//    sums are integers (mass x 2^S rounded, 64-bit atomics), so the image does not depend on the
//    order the atomics land in; S leaves headroom for the total mass.
//  - Tone map: reference level = mean lit pixel value, white point = 99.5th percentile of the lit
//    pixels (radix select), t = log1p(m / ref) / log1p(white / ref), the reference's colour ramps.
#include <cfloat>
#include <cmath>
#include <cstdlib>
#include <cstring>
#include <string>
#include <vector>

#include "engine.cuh"

namespace lg {

namespace {

constexpr int RBS = 256;
inline int grid_for(long long n, int bs) { return static_cast<int>((n + bs - 1) / bs); }

struct Proj {
    double ax[3], ay[3];
};

Proj parse_view(const std::string& view) {
    if (view == "xy") return {{1, 0, 0}, {0, 1, 0}};
    if (view == "xz") return {{1, 0, 0}, {0, 0, 1}};
    if (view == "yz") return {{0, 1, 0}, {0, 0, 1}};
    const size_t comma = view.find(',');
    auto bad = [&]() { fail(kArg, "bad view '" + view + "': expected xy|xz|yz|<yaw>,<pitch>"); };
    if (comma == std::string::npos) bad();
    const std::string a = view.substr(0, comma), b = view.substr(comma + 1);
    char *ea = nullptr, *eb = nullptr;
    const double yaw = std::strtod(a.c_str(), &ea), pitch = std::strtod(b.c_str(), &eb);
    auto only_space = [](const char* p) {
        while (*p == ' ' || *p == '\t') ++p;
        return *p == 0;
    };
    if (a.empty() || b.empty() || !only_space(ea) || !only_space(eb) || !std::isfinite(yaw) || !std::isfinite(pitch))
        bad();
    const double k = 3.14159265358979323846 / 180;
    const double cy = std::cos(yaw * k), sy = std::sin(yaw * k), cp = std::cos(pitch * k), sp = std::sin(pitch * k);
    // Rotate about z by yaw, then about x by pitch.
    return {{cy, -sy, 0}, {cp * sy, cp * cy, -sp}};
}

struct RenderArgs {
    const float4* hm;
    const float* vx;
    const float* vy;
    const float* vz;
    int n, W, H, speed;
    double ax0, ax1, ax2, ay0, ay1, ay2;
};

__device__ __forceinline__ void project(const RenderArgs& a, int i, double& sx, double& sy, float& m, float& sp,
                                        bool& ok) {
    const float4 h = a.hm[i];
    sx = a.ax0 * h.x + a.ax1 * h.y + a.ax2 * h.z;
    sy = a.ay0 * h.x + a.ay1 * h.y + a.ay2 * h.z;
    m = h.w;
    sp = 0.f;
    if (a.speed) {
        const float x = a.vx[i], y = a.vy[i], z = a.vz[i];
        sp = sqrtf(x * x + y * y + z * z);
    }
    ok = isfinite(sx) && isfinite(sy) && isfinite(m) && (!a.speed || isfinite(sp));
}

// Block FP64 sums of (mass, mass sx, mass sy, mass v^2, finite count) into out[5] with atomics.
__global__ void k_render_moments(RenderArgs a, double* out) {
    __shared__ double sh[5][RBS / 32];
    double v[5] = {0, 0, 0, 0, 0};
    for (int i = blockIdx.x * RBS + threadIdx.x; i < a.n; i += gridDim.x * RBS) {
        double sx, sy;
        float m, sp;
        bool ok;
        project(a, i, sx, sy, m, sp, ok);
        if (!ok) continue;
        v[0] += m;
        v[1] += m * sx;
        v[2] += m * sy;
        if (a.speed) v[3] += static_cast<double>(m) * (static_cast<double>(sp) * sp);
        v[4] += 1.0;
    }
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
#pragma unroll
    for (int k = 0; k < 5; ++k) {
        for (int o = 16; o > 0; o >>= 1) v[k] += __shfl_down_sync(0xffffffffu, v[k], o);
        if (lane == 0) sh[k][w] = v[k];
    }
    __syncthreads();
    if (threadIdx.x < 5) {
        double s = 0;
        for (int u = 0; u < RBS / 32; ++u) s += sh[threadIdx.x][u];
        atomicAdd(out + threadIdx.x, s);
    }
}

// Distances from the centre as float bits (non-finite bodies: 0xffffffff, never selected).
__global__ void k_render_dist(RenderArgs a, double cx, double cy, uint32_t* bits) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= a.n) return;
    double sx, sy;
    float m, sp;
    bool ok;
    project(a, i, sx, sy, m, sp, ok);
    bits[i] = ok ? __float_as_uint(static_cast<float>(hypot(sx - cx, sy - cy))) : 0xffffffffu;
}

// Radix select, one 8-bit digit per pass: histogram of the values whose higher digits equal prefix.
__global__ void k_select_hist(const uint32_t* __restrict__ v, size_t n, uint32_t prefix, uint32_t mask, int shift,
                              unsigned* hist) {
    __shared__ unsigned h[256];
    for (int k = threadIdx.x; k < 256; k += blockDim.x) h[k] = 0;
    __syncthreads();
    for (size_t i = blockIdx.x * static_cast<size_t>(blockDim.x) + threadIdx.x; i < n;
         i += static_cast<size_t>(gridDim.x) * blockDim.x) {
        const uint32_t x = v[i];
        if ((x & mask) == prefix) atomicAdd(&h[(x >> shift) & 255u], 1u);
    }
    __syncthreads();
    for (int k = threadIdx.x; k < 256; k += blockDim.x)
        if (h[k]) atomicAdd(&hist[k], h[k]);
}

// Fixed-point bilinear splat: mass (and mass x speed) x 2^S into 64-bit pixel sums.
__global__ void k_render_splat(RenderArgs a, double cx, double cy, double scale, double s_m, double s_v,
                               unsigned long long* img) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= a.n) return;
    double sx, sy;
    float m, sp;
    bool ok;
    project(a, i, sx, sy, m, sp, ok);
    if (!ok) return;
    const int W = a.W, H = a.H, ch = a.speed ? 2 : 1;
    const double px = (sx - cx) * scale + W * 0.5 - 0.5;
    const double py = H * 0.5 - (sy - cy) * scale - 0.5;
    const double fx0 = floor(px), fy0 = floor(py);
    if (!(fx0 > -2 && fx0 < W + 1 && fy0 > -2 && fy0 < H + 1)) return;
    const int ix = static_cast<int>(fx0), iy = static_cast<int>(fy0);
    const float fx = static_cast<float>(px - fx0), fy = static_cast<float>(py - fy0);
    const float mv = a.speed ? m * sp : 0.f;
    const float w[4] = {(1 - fx) * (1 - fy), fx * (1 - fy), (1 - fx) * fy, fx * fy};
#pragma unroll
    for (int k = 0; k < 4; ++k) {
        const int xx = ix + (k & 1), yy = iy + (k >> 1);
        if (xx >= 0 && xx < W && yy >= 0 && yy < H) {
            const size_t p = (static_cast<size_t>(yy) * W + xx) * ch;
            atomicAdd(img + p, static_cast<unsigned long long>(llrint(static_cast<double>(m * w[k]) * s_m)));
            if (a.speed)
                atomicAdd(img + p + 1, static_cast<unsigned long long>(llrint(static_cast<double>(mv * w[k]) * s_v)));
        }
    }
}

// Fixed point to float pixels; lit pixels' float bits for the white-point select (unlit: ~0);
// FP64 sum of the lit values and their count.
__global__ void k_render_unfix(const unsigned long long* __restrict__ img, size_t npix, int ch, double inv_m,
                               double inv_v, float* out, uint32_t* lit, double* sum) {
    __shared__ double sh[2][RBS / 32];
    double s = 0, c = 0;
    for (size_t p = blockIdx.x * static_cast<size_t>(RBS) + threadIdx.x; p < npix;
         p += static_cast<size_t>(gridDim.x) * RBS) {
        // Two's-complement sums: signed, so that negative masses would still add up.
        const float v = static_cast<float>(static_cast<double>(static_cast<long long>(img[p * ch])) * inv_m);
        out[p * ch] = v;
        if (ch == 2)
            out[p * ch + 1] = static_cast<float>(static_cast<double>(static_cast<long long>(img[p * ch + 1])) * inv_v);
        lit[p] = v > 0.f ? __float_as_uint(v) : 0xffffffffu;
        if (v > 0.f) {
            s += v;
            c += 1.0;
        }
    }
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    for (int o = 16; o > 0; o >>= 1) {
        s += __shfl_down_sync(0xffffffffu, s, o);
        c += __shfl_down_sync(0xffffffffu, c, o);
    }
    if (lane == 0) {
        sh[0][w] = s;
        sh[1][w] = c;
    }
    __syncthreads();
    if (threadIdx.x < 2) {
        double t = 0;
        for (int u = 0; u < RBS / 32; ++u) t += sh[threadIdx.x][u];
        atomicAdd(sum + threadIdx.x, t);
    }
}

struct Rgb {
    float r, g, b;
};

__device__ Rgb ramp4(float t, const float (&st)[4], const float (&c)[4][3]) {
    t = fminf(fmaxf(t, 0.f), 1.f);
    for (int i = 1; i < 4; ++i)
        if (t <= st[i]) {
            const float u = (t - st[i - 1]) / (st[i] - st[i - 1]);
            return {c[i - 1][0] + u * (c[i][0] - c[i - 1][0]), c[i - 1][1] + u * (c[i][1] - c[i - 1][1]),
                    c[i - 1][2] + u * (c[i][2] - c[i - 1][2])};
        }
    return {c[3][0], c[3][1], c[3][2]};
}

// The reference's colour ramps (src/render.cpp:43-70).
__device__ Rgb density_ramp(float t) {
    const float st[4] = {0.00f, 0.35f, 0.70f, 1.00f};
    const float c[4][3] = {{10, 12, 70}, {120, 30, 150}, {255, 140, 30}, {255, 255, 255}};
    return ramp4(t, st, c);
}

__device__ Rgb speed_ramp(float t) {
    const float st[4] = {0.00f, 0.40f, 0.70f, 1.00f};
    const float c[4][3] = {{40, 90, 255}, {80, 230, 255}, {255, 230, 90}, {255, 60, 40}};
    return ramp4(t, st, c);
}

__global__ void k_render_tone(const float* __restrict__ img, size_t npix, int ch, float vref, float norm,
                              float vref_speed, unsigned char* rgb) {
    const size_t p = blockIdx.x * static_cast<size_t>(blockDim.x) + threadIdx.x;
    if (p >= npix) return;
    const float m = img[p * ch];
    unsigned char r = 0, g = 0, b = 0;
    if (m > 0) {
        const float t = log1pf(m / vref) * norm;
        Rgb c;
        if (ch == 2) {
            const Rgb h = speed_ramp(img[p * ch + 1] / m / vref_speed);
            const float k = 0.25f + 0.75f * t;
            c = {h.r * k, h.g * k, h.b * k};
        } else {
            c = density_ramp(t);
        }
        r = static_cast<unsigned char>(c.r + 0.5f);
        g = static_cast<unsigned char>(c.g + 0.5f);
        b = static_cast<unsigned char>(c.b + 0.5f);
    }
    rgb[3 * p] = r;
    rgb[3 * p + 1] = g;
    rgb[3 * p + 2] = b;
}

// k-th smallest (0-based) of n uint32 values on the device, four 8-bit passes (host-driven).
uint32_t radix_select(Engine& e, const uint32_t* v, size_t n, size_t k, DevBuf& hist) {
    hist.reserve(256 * 4);
    uint32_t prefix = 0, mask = 0;
    unsigned* h = e.pinned_small + 256;
    const int blocks = std::max(1, std::min(4 * e.sms, grid_for(static_cast<long long>(n), RBS)));
    for (int shift = 24; shift >= 0; shift -= 8) {
        LG_CK(cudaMemsetAsync(hist.as<unsigned>(), 0, 256 * 4, e.stream));
        k_select_hist<<<blocks, RBS, 0, e.stream>>>(v, n, prefix, mask, shift, hist.as<unsigned>());
        LG_LAUNCHED();
        ++e.launches;
        LG_CK(cudaMemcpyAsync(h, hist.as<unsigned>(), 256 * 4, cudaMemcpyDeviceToHost, e.stream));
        LG_CK(cudaStreamSynchronize(e.stream));
        uint32_t d = 0;
        for (; d < 256; ++d) {
            if (k < h[d]) break;
            k -= h[d];
        }
        if (d == 256) d = 255;
        prefix |= d << shift;
        mask |= 255u << shift;
    }
    return prefix;
}

}  // namespace

void render(Engine& e, const lg_render_options& o, unsigned char* rgb, double* extent_used) {
    if (o.width < 1 || o.height < 1 || o.width > 65536 || o.height > 65536) fail(kArg, "render: bad image size");
    if (!(o.extent >= 0)) fail(kArg, "render: extent must be >= 0");
    const Proj P = parse_view(o.view ? std::string(o.view) : std::string("xy"));
    const int W = o.width, H = o.height, n = e.n;
    const bool speed = o.color == 1;
    const int ch = speed ? 2 : 1;
    const size_t npix = static_cast<size_t>(W) * H;
    cudaStream_t s = e.stream;
    const BodyArrays b = e.bodies(e.cur);
    RenderArgs a{b.hm, b.vx, b.vy, b.vz, n, W, H, speed ? 1 : 0, P.ax[0], P.ax[1], P.ax[2], P.ay[0], P.ay[1], P.ay[2]};
    // Moments of the finite bodies.
    double* mom = e.dscratch();
    LG_CK(cudaMemsetAsync(mom, 0, 5 * 8, s));
    if (n > 0) {
        k_render_moments<<<std::max(1, std::min(2 * e.sms, grid_for(n, RBS))), RBS, 0, s>>>(a, mom);
        LG_LAUNCHED();
        ++e.launches;
    }
    double hm[5];
    LG_CK(cudaMemcpyAsync(hm, mom, 5 * 8, cudaMemcpyDeviceToHost, s));
    LG_CK(cudaStreamSynchronize(s));
    const double mtot = hm[0];
    double cx = 0, cy = 0;
    if (mtot > 0) {
        cx = hm[1] / mtot;
        cy = hm[2] / mtot;
    }
    const float vref_speed = mtot > 0 && hm[3] > 0 ? static_cast<float>(2 * std::sqrt(hm[3] / mtot)) : 1.f;
    const size_t m = static_cast<size_t>(hm[4]);
    DevBuf& bits = e.partial;  // scratch: n distances, then the lit pixels
    DevBuf hist;
    double extent = o.extent;
    if (extent == 0) {
        if (m > 0) {
            bits.reserve(std::max(static_cast<size_t>(n), npix) * 4 + 16);
            k_render_dist<<<grid_for(n, RBS), RBS, 0, s>>>(a, cx, cy, bits.as<uint32_t>());
            LG_LAUNCHED();
            ++e.launches;
            const size_t k = std::min(m - 1, static_cast<size_t>(0.99 * static_cast<double>(m)));
            const uint32_t d = radix_select(e, bits.as<uint32_t>(), static_cast<size_t>(n), k, hist);
            float df;
            std::memcpy(&df, &d, 4);
            extent = 1.2 * df;
        }
        if (!(extent > 0)) extent = 1;
    }
    const double scale = W / (2 * extent);
    // Fixed-point scales: any pixel sum stays below 2^62.
    const double s_m = mtot > 0 ? std::ldexp(1.0, 61 - std::ilogb(mtot) - 1) : 1.0;
    double vmass = 0;
    if (speed && mtot > 0) vmass = std::sqrt(hm[3] * mtot);  // Cauchy-Schwarz bound of sum m |v|
    const double s_v = vmass > 0 ? std::ldexp(1.0, 61 - std::ilogb(vmass) - 1) : 1.0;
    DevBuf& fix = e.vjp_scratch;
    fix.reserve(npix * ch * 8);
    LG_CK(cudaMemsetAsync(fix.as<char>(), 0, npix * ch * 8, s));
    if (n > 0) {
        k_render_splat<<<grid_for(n, RBS), RBS, 0, s>>>(a, cx, cy, scale, s_m, s_v, fix.as<unsigned long long>());
        LG_LAUNCHED();
        ++e.launches;
    }
    DevBuf& fimg = e.staging;
    fimg.reserve(npix * ch * 4);
    bits.reserve(std::max(static_cast<size_t>(n), npix) * 4 + 16);
    LG_CK(cudaMemsetAsync(mom, 0, 2 * 8, s));
    k_render_unfix<<<std::max(1, std::min(4 * e.sms, grid_for(static_cast<long long>(npix), RBS))), RBS, 0, s>>>(
        fix.as<unsigned long long>(), npix, ch, 1.0 / s_m, 1.0 / s_v, fimg.as<float>(), bits.as<uint32_t>(), mom);
    LG_LAUNCHED();
    ++e.launches;
    LG_CK(cudaMemcpyAsync(hm, mom, 2 * 8, cudaMemcpyDeviceToHost, s));
    LG_CK(cudaStreamSynchronize(s));
    const size_t nz = static_cast<size_t>(hm[1]);
    DevBuf out;
    out.reserve(npix * 3);
    if (nz > 0) {
        const size_t k = std::min(nz - 1, static_cast<size_t>(0.995 * static_cast<double>(nz)));
        const uint32_t vb = radix_select(e, bits.as<uint32_t>(), npix, k, hist);
        float vmax;
        std::memcpy(&vmax, &vb, 4);
        const float vref = static_cast<float>(hm[0] / static_cast<double>(nz));
        const float norm = 1.f / std::max(std::log1p(vmax / vref), 1e-6f);
        k_render_tone<<<grid_for(static_cast<long long>(npix), RBS), RBS, 0, s>>>(fimg.as<float>(), npix, ch, vref, norm,
                                                                               vref_speed, out.as<unsigned char>());
        LG_LAUNCHED();
        ++e.launches;
    } else {
        LG_CK(cudaMemsetAsync(out.as<char>(), 0, npix * 3, s));
    }
    LG_CK(cudaMemcpyAsync(rgb, out.as<unsigned char>(), npix * 3, cudaMemcpyDeviceToHost, s));
    LG_CK(cudaStreamSynchronize(s));
    if (extent_used) *extent_used = extent;
}

}  // namespace lg
