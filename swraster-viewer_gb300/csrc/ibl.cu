// Load-time texture precompute on the device (see ibl.h): mip chains, the
// BRDF LUT and the GGX-prefiltered environment, bit-exact with the host
// restatement in scene.cpp. Built with -fmad=false like every kernel here:
// each multiply and add rounds on its own, as in the reference.
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstring>

#include "ibl.h"

namespace swr {

namespace {

// Half-width, in ulps, of the interval the GGX prefilter takes around the
// device's powf: it must hold the host libm's powf for every input.
// tests/test_ibl_device.py compares the two functions over every float the
// inputs can take and requires their difference to stay within it (the
// largest difference measured on GB300 against glibc is 1 ulp).
constexpr int kPowUlps = 2;

struct F3 {
    float x, y, z;
};
__device__ __forceinline__ F3 f3add(F3 a, F3 b) { return {a.x + b.x, a.y + b.y, a.z + b.z}; }
__device__ __forceinline__ F3 f3sub(F3 a, F3 b) { return {a.x - b.x, a.y - b.y, a.z - b.z}; }
__device__ __forceinline__ F3 f3mul(F3 a, float s) { return {a.x * s, a.y * s, a.z * s}; }
// Vec3A::dot (x*x' + y*y') + z*z'; normalize = self * (1 / length).
__device__ __forceinline__ float f3dot(F3 a, F3 b) { return (a.x * b.x + a.y * b.y) + a.z * b.z; }
__device__ __forceinline__ F3 f3norm(F3 a) { return f3mul(a, 1.0f / sqrtf(f3dot(a, a))); }
__device__ __forceinline__ F3 f3cross(F3 a, F3 b) {
    return {a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x};
}

// rgba8_unpack_vec4 / rgba8_pack_vec4 (src/util.rs:83-96); `as u32` saturates.
__device__ __forceinline__ float byte_unit(uint32_t c, int shift) { return (float)((c >> shift) & 0xFFu) / 255.0f; }
__device__ __forceinline__ uint32_t sat_u32(float x) {
    if (!(x > 0.0f)) return 0u;
    if (x >= 4294967296.0f) return 0xFFFFFFFFu;
    return (uint32_t)x;
}
__device__ __forceinline__ uint32_t to_byte(float c) { return sat_u32(c * 255.0f); }
__device__ __forceinline__ uint32_t pack_bytes(uint32_t r, uint32_t g, uint32_t b, uint32_t a) {
    return (r << 24) | (g << 16) | (b << 8) | a;
}

// The powf calls of the tables, shared with the self-test.
__device__ __forceinline__ float pow_24(float x) { return powf(x, 2.4f); }
__device__ __forceinline__ float pow_inv24(float x) { return powf(x, 1.0f / 2.4f); }
// [p - kPowUlps ulp, p + kPowUlps ulp] for a positive normal p.
__device__ __forceinline__ void widen(float p, float& lo, float& hi) {
    const int b = __float_as_int(p);
    lo = __int_as_float(b - kPowUlps);
    hi = __int_as_float(b + kPowUlps);
}

// srgb_to_linear_scalar (src/util.rs:49-55) of an interpolated value: the
// host's result lies in [lo, hi].
__device__ __forceinline__ void srgb_to_linear_iv(float s, float& lo, float& hi) {
    if (s <= 0.04045f) {
        lo = hi = s / 12.92f;
        return;
    }
    const float x = (s + 0.055f) / 1.055f;
    // powf(1, y) is exactly 1 in every conforming libm (C11 F.10.4.4): white
    // samples stay exact.
    if (x == 1.0f) {
        lo = hi = 1.0f;
        return;
    }
    widen(pow_24(x), lo, hi);
}

// The byte linear_to_srgb_scalar (src/util.rs:66-72) packs to. Its powf
// branch goes through the host's byte thresholds: thr[k - 1] is the smallest
// float whose byte is at least k, so the byte is the number of thresholds
// at or below s (the host's byte is non-decreasing in s; the tests check it
// over every float of the branch).
__device__ __forceinline__ uint32_t linear_to_srgb_byte(float s, const float* __restrict__ thr) {
    if (s <= 0.0031308f) return to_byte(s * 12.92f);
    uint32_t lo = 0, hi = 255;  // count of thresholds <= s lies in [lo, hi]
    while (lo < hi) {
        const uint32_t mid = (lo + hi + 1) >> 1;
        if (__ldg(thr + mid - 1) <= s) lo = mid;
        else hi = mid - 1;
    }
    return lo;
}

// One texel of the next mip (src/texture.rs:82-113). s2l: the 256 values of
// srgb_to_linear_scalar(b / 255) as the host computes them; thr: the byte
// thresholds of linear_to_srgb_byte.
__device__ uint32_t mip_texel_dev(uint32_t type, uint32_t q00, uint32_t q10, uint32_t q01, uint32_t q11,
                                  const float* __restrict__ s2l, const float* __restrict__ thr) {
    const int sh[4] = {24, 16, 8, 0};
    uint32_t out[4];
    if (type == SWR_TEX_SRGB) {
        for (int c = 0; c < 3; ++c) {
            const float l00 = __ldg(s2l + ((q00 >> sh[c]) & 0xFFu)), l10 = __ldg(s2l + ((q10 >> sh[c]) & 0xFFu));
            const float l01 = __ldg(s2l + ((q01 >> sh[c]) & 0xFFu)), l11 = __ldg(s2l + ((q11 >> sh[c]) & 0xFFu));
            const float s = (((l00 + l10) + l01) + l11) / 4.0f;
            out[c] = linear_to_srgb_byte(s, thr);
        }
        const float w = (((byte_unit(q00, 0) + byte_unit(q10, 0)) + byte_unit(q01, 0)) + byte_unit(q11, 0)) / 4.0f;
        out[3] = to_byte(w);
    } else if (type == SWR_TEX_METALLIC_ROUGHNESS) {
        const float y00 = byte_unit(q00, 16), y10 = byte_unit(q10, 16), y01 = byte_unit(q01, 16),
                    y11 = byte_unit(q11, 16);
        const float r = (((y00 * y00 + y10 * y10) + y01 * y01) + y11 * y11) / 4.0f;
        const float m = (((byte_unit(q00, 8) + byte_unit(q10, 8)) + byte_unit(q01, 8)) + byte_unit(q11, 8)) / 4.0f;
        out[0] = to_byte(byte_unit(q00, 24));
        out[1] = to_byte(sqrtf(r));
        out[2] = to_byte(m);
        out[3] = to_byte(byte_unit(q00, 0));
    } else if (type == SWR_TEX_NORMAL) {
        for (int c = 0; c < 4; ++c) {
            const float n00 = byte_unit(q00, sh[c]) * 2.0f - 1.0f, n10 = byte_unit(q10, sh[c]) * 2.0f - 1.0f;
            const float n01 = byte_unit(q01, sh[c]) * 2.0f - 1.0f, n11 = byte_unit(q11, sh[c]) * 2.0f - 1.0f;
            const float s = (((n00 + n10) + n01) + n11) / 4.0f;
            out[c] = to_byte((s + 1.0f) / 2.0f);
        }
    } else {
        for (int c = 0; c < 4; ++c) {
            const float s = ((byte_unit(q00, sh[c]) + byte_unit(q10, sh[c])) + byte_unit(q01, sh[c])) +
                            byte_unit(q11, sh[c]);
            out[c] = to_byte(s / 4.0f);
        }
    }
    return pack_bytes(out[0], out[1], out[2], out[3]);
}

struct MipJob {
    const uint32_t* src;  // previous level
    uint32_t* dst;        // this level
    uint32_t pw, ph, pstride, mw, mh, slices, type;
};

// One mip level.
__global__ void k_mip(MipJob j, const float* __restrict__ s2l, const float* __restrict__ thr) {
    const uint32_t plane = j.mw * j.mh;
    const uint32_t n = plane * j.slices;
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        const uint32_t slice = i / plane, rem = i - slice * plane;
        const uint32_t y = rem / j.mw, x = rem - y * j.mw;
        const uint32_t x0 = x * 2, y0 = y * 2;
        const uint32_t x1 = min(x0 + 1, j.pw - 1), y1 = min(y0 + 1, j.ph - 1);
        const uint32_t* s = j.src + (size_t)slice * j.pstride;
        const uint32_t q00 = s[y0 * j.pw + x0], q10 = s[y0 * j.pw + x1];
        const uint32_t q01 = s[y1 * j.pw + x0], q11 = s[y1 * j.pw + x1];
        j.dst[i] = mip_texel_dev(j.type, q00, q10, q01, q11, s2l, thr);
    }
}

// importance_sample_ggx (src/texture.rs:148-167); the sample's angle enters
// as its cosine and sine, computed on the host.
__device__ __forceinline__ F3 ggx_sample(float xi_y, float cos_phi, float sin_phi, F3 n, float roughness) {
    const float a = roughness * roughness;
    const float cos_theta = sqrtf((1.0f - xi_y) / (1.0f + (a * a - 1.0f) * xi_y));
    const float sin_theta = sqrtf(fmaxf(1.0f - cos_theta * cos_theta, 0.0f));
    const F3 h = {cos_phi * sin_theta, sin_phi * sin_theta, cos_theta};
    const F3 up = fabsf(n.z) < 0.999f ? F3{0.0f, 0.0f, 1.0f} : F3{1.0f, 0.0f, 0.0f};
    const F3 tangent = f3norm(f3cross(n, up));
    const F3 bitangent = f3cross(n, tangent);
    return f3norm(f3add(f3add(f3mul(tangent, h.x), f3mul(bitangent, h.y)), f3mul(n, h.z)));
}

// generate_brdf_lut + integrate_brdf (src/texture.rs:169-243); samp[i] =
// (xi_x, xi_y, cos, sin) of hammersley(i, 128).
__global__ void k_brdf(uint32_t size, const float4* __restrict__ samp, uint32_t* __restrict__ out) {
    const uint32_t n = size * size;
    const float size_f = (float)size;
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        const uint32_t y = i / size, x = i - y * size;
        const float roughness_c = fminf(fmaxf(((float)y + 0.5f) / size_f, 0.0f), 1.0f);
        const float ndotv_c = fminf(fmaxf(((float)x + 0.5f) / size_f, 0.0f), 1.0f);
        const float ndotv = fmaxf(ndotv_c, 1.0e-4f), roughness = fmaxf(roughness_c, 1.0e-4f);
        const F3 v = {sqrtf(fmaxf(1.0f - ndotv * ndotv, 0.0f)), 0.0f, ndotv};
        const F3 nz = {0.0f, 0.0f, 1.0f};
        float ra = 0.0f, rb = 0.0f;
        for (uint32_t s = 0; s < 128; ++s) {
            const float4 q = __ldg(samp + s);
            const F3 h = ggx_sample(q.y, q.z, q.w, nz, roughness);
            const F3 l = f3norm(f3sub(f3mul(h, 2.0f * f3dot(v, h)), v));
            const float ndotl = fmaxf(l.z, 0.0f);
            const float ndoth = fmaxf(h.z, 0.0f);
            const float vdoth = fmaxf(f3dot(v, h), 0.0f);
            if (ndotl > 0.0f) {
                const float alpha = roughness * roughness;
                const float k = ((alpha + 1.0f) * (alpha + 1.0f)) * 0.125f;
                const float g_v = ndotv / (ndotv * (1.0f - k) + k);
                const float g_l = ndotl / (ndotl * (1.0f - k) + k);
                const float g_vis = fmaxf(((g_v * g_l) * vdoth) / (ndoth * fmaxf(ndotv, 1.0e-5f)), 0.0f);
                const float o = 1.0f - vdoth;
                const float o2 = o * o;
                const float fc = o * (o2 * o2);  // powi(5)
                ra += (1.0f - fc) * g_vis;
                rb += fc * g_vis;
            }
        }
        const float ia = ra / 128.0f, ib = rb / 128.0f;
        out[i] = pack_bytes(to_byte(fminf(fmaxf(ia, 0.0f), 1.0f)), to_byte(fminf(fmaxf(ib, 0.0f), 1.0f)), 0u,
                            to_byte(1.0f));
    }
}

// cubemap_face_uv_to_direction / cubemap_direction_to_face_uv
// (src/texture.rs:245-271).
__device__ __forceinline__ F3 face_dir(uint32_t face, float u, float v) {
    F3 d;
    switch (face) {
        case 0: d = {1.0f, -v, -u}; break;
        case 1: d = {-1.0f, -v, u}; break;
        case 2: d = {u, 1.0f, v}; break;
        case 3: d = {u, -1.0f, -v}; break;
        case 4: d = {u, -v, 1.0f}; break;
        default: d = {-u, -v, -1.0f}; break;
    }
    return f3norm(d);
}
__device__ __forceinline__ void dir_face_uv(F3 n, uint32_t& face, float& u, float& v) {
    const float ax = fabsf(n.x), ay = fabsf(n.y), az = fabsf(n.z);
    if (ax >= ay && ax >= az) {
        if (n.x >= 0.0f) { face = 0; u = (-n.z / ax) * 0.5f + 0.5f; v = (-n.y / ax) * 0.5f + 0.5f; }
        else { face = 1; u = (n.z / ax) * 0.5f + 0.5f; v = (-n.y / ax) * 0.5f + 0.5f; }
    } else if (ay > ax && ay >= az) {
        if (n.y >= 0.0f) { face = 2; u = (n.x / ay) * 0.5f + 0.5f; v = (n.z / ay) * 0.5f + 0.5f; }
        else { face = 3; u = (n.x / ay) * 0.5f + 0.5f; v = (-n.z / ay) * 0.5f + 0.5f; }
    } else if (n.z >= 0.0f) {
        face = 4; u = (n.x / az) * 0.5f + 0.5f; v = (-n.y / az) * 0.5f + 0.5f;
    } else {
        face = 5; u = (-n.x / az) * 0.5f + 0.5f; v = (-n.y / az) * 0.5f + 0.5f;
    }
}

struct Cube {
    const uint32_t* data;  // mip 0, six faces of w x h
    uint32_t w, h;
};

// sample_cubemap_direction_linear (src/texture.rs:273-287): bilinear lane 0
// with ClampToEdge at mip 0 (src/texture.rs:730-790), then to linear; the
// host's value of each channel lies in [lo, hi].
__device__ void sample_dir_iv(const Cube& c, F3 dir, F3& lo, F3& hi) {
    uint32_t face;
    float u, v;
    dir_face_uv(dir, face, u, v);
    u = fminf(fmaxf(u, 0.0f), 1.0f);
    v = fminf(fmaxf(v, 0.0f), 1.0f);
    const float wf = (float)c.w, hf = (float)c.h;
    const uint32_t* base = c.data + (size_t)face * c.w * c.h;
    const float xf = u * wf - 0.5f, yf = v * hf - 0.5f;
    const float x0 = floorf(xf), y0 = floorf(yf);
    const float x1 = x0 + 1.0f, y1 = y0 + 1.0f;
    const float fx = xf - x0, fy = yf - y0;
    const float ofx = 1.0f - fx, ofy = 1.0f - fy;
    const uint32_t x0i = sat_u32(fminf(x0, wf - 1.0f)), y0i = sat_u32(fminf(y0, hf - 1.0f));
    const uint32_t x1i = sat_u32(fminf(x1, wf - 1.0f)), y1i = sat_u32(fminf(y1, hf - 1.0f));
    const uint32_t p00 = __ldg(base + y0i * c.w + x0i), p10 = __ldg(base + y0i * c.w + x1i);
    const uint32_t p01 = __ldg(base + y1i * c.w + x0i), p11 = __ldg(base + y1i * c.w + x1i);
    const float w00 = ofx * ofy, w10 = fx * ofy, w01 = ofx * fy, w11 = fx * fy;
    float s[3];
    const int sh[3] = {24, 16, 8};
    for (int k = 0; k < 3; ++k)
        s[k] = ((byte_unit(p00, sh[k]) * w00 + byte_unit(p10, sh[k]) * w10) + byte_unit(p01, sh[k]) * w01) +
               byte_unit(p11, sh[k]) * w11;
    srgb_to_linear_iv(s[0], lo.x, hi.x);
    srgb_to_linear_iv(s[1], lo.y, hi.y);
    srgb_to_linear_iv(s[2], lo.z, hi.z);
}

struct PrefilterArgs {
    Cube cube;
    uint32_t max_mip, samples;
    const float4* samp;  // (xi_x, xi_y, cos, sin) of hammersley(i, samples)
    uint32_t* out;       // (max_mip + 1) x 6 faces x w x h
    uint32_t* flags;     // texel indices left open
    uint32_t* nflags;
};

// generate_prefiltered_specular_cubemap (src/texture.rs:330-420), one thread
// per output texel. The sums of positive terms, the division by the positive
// total and the byte conversion are monotone, so running them on the
// interval's lower and upper ends brackets the host's texel.
__global__ void k_prefilter(PrefilterArgs a) {
    const uint32_t w = a.cube.w, h = a.cube.h;
    const uint32_t face_texels = w * h;
    const uint64_t n = (uint64_t)face_texels * 6u * (a.max_mip + 1u);
    for (uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; i < n; i += (uint64_t)gridDim.x * blockDim.x) {
        const uint32_t mip = (uint32_t)(i / (6ull * face_texels));
        const uint32_t rem = (uint32_t)(i - (uint64_t)mip * 6u * face_texels);
        const uint32_t face = rem / face_texels;
        const uint32_t t = rem - face * face_texels;
        const uint32_t y = t / w, x = t - y * w;
        const float roughness = a.max_mip > 0 ? (float)mip / (float)a.max_mip : 0.0f;
        const float v = (((float)y + 0.5f) / (float)h) * 2.0f - 1.0f;
        const float u = (((float)x + 0.5f) / (float)w) * 2.0f - 1.0f;
        const F3 r = face_dir(face, u, v);
        F3 lo, hi;
        bool direct = mip == 0;
        if (!direct) {
            F3 acc_lo = {0.0f, 0.0f, 0.0f}, acc_hi = {0.0f, 0.0f, 0.0f};
            float total = 0.0f;
            const float rough = fmaxf(roughness, 0.045f);
            for (uint32_t s = 0; s < a.samples; ++s) {
                const float4 q = __ldg(a.samp + s);
                const F3 hv = ggx_sample(q.y, q.z, q.w, r, rough);
                const F3 l = f3norm(f3sub(f3mul(hv, 2.0f * f3dot(r, hv)), r));
                const float ndotl = fmaxf(f3dot(r, l), 0.0f);
                if (ndotl > 0.0f) {
                    F3 clo, chi;
                    sample_dir_iv(a.cube, l, clo, chi);
                    acc_lo = f3add(acc_lo, f3mul(clo, ndotl));
                    acc_hi = f3add(acc_hi, f3mul(chi, ndotl));
                    total += ndotl;
                }
            }
            if (total > 0.0f) {
                lo = {acc_lo.x / total, acc_lo.y / total, acc_lo.z / total};
                hi = {acc_hi.x / total, acc_hi.y / total, acc_hi.z / total};
            } else {
                direct = true;
            }
        }
        if (direct) sample_dir_iv(a.cube, r, lo, hi);
        const uint32_t br = to_byte(lo.x), bg = to_byte(lo.y), bb = to_byte(lo.z);
        a.out[i] = pack_bytes(br, bg, bb, to_byte(1.0f));
        if (br != to_byte(hi.x) || bg != to_byte(hi.y) || bb != to_byte(hi.z)) {
            const uint32_t k = atomicAdd(a.nflags, 1u);
            a.flags[k] = (uint32_t)i;
        }
    }
}

__global__ void k_pow_selftest(const float* in, float* out, uint64_t n, uint32_t mode) {
    for (uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; i < n; i += (uint64_t)gridDim.x * blockDim.x)
        out[i] = mode == 0 ? pow_24(in[i]) : pow_inv24(in[i]);
}

// Device allocations freed on every return path.
struct Mem {
    std::vector<void*> ptrs;
    ~Mem() {
        for (void* p : ptrs) cudaFree(p);
    }
    template <class T>
    cudaError_t alloc(T** p, size_t count) {
        void* q = nullptr;
        const cudaError_t e = cudaMalloc(&q, std::max<size_t>(count, 1) * sizeof(T));
        if (e == cudaSuccess) ptrs.push_back(q);
        *p = static_cast<T*>(q);
        return e;
    }
};

uint32_t grid_for(uint64_t n, uint32_t threads) {
    int dev = 0, sms = 1;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    const uint64_t want = (n + threads - 1) / threads;
    return (uint32_t)std::max<uint64_t>(1, std::min<uint64_t>(want, (uint64_t)sms * 16));
}

swr_status cuda_status(cudaError_t e, const char* what, std::string& err) {
    err = std::string(what) + ": " + cudaGetErrorString(e);
    cudaGetLastError();
    return e == cudaErrorMemoryAllocation ? SWR_NO_MEMORY : SWR_CUDA_ERROR;
}

}  // namespace

swr_status mipmaps_device(const std::vector<HTexture*>& textures, std::string& err) {
    size_t max_total = 0;
    for (HTexture* t : textures) {
        t->mip_layout();
        const uint32_t slices = t->type == SWR_TEX_CUBEMAP ? 6u : 1u;
        const size_t total = (size_t)t->mip_offsets[t->max_mip] +
                             (size_t)t->mip_widths[t->max_mip] * t->mip_heights[t->max_mip] * slices;
        max_total = std::max(max_total, total);
    }
    float s2l_host[256], thr_host[255];
    for (int b = 0; b < 256; ++b) s2l_host[b] = srgb_to_linear_host((float)b / 255.0f);
    srgb_byte_thresholds(thr_host);
    Mem m;
    uint32_t* d_data = nullptr;
    float *d_s2l = nullptr, *d_thr = nullptr;
    cudaError_t e = m.alloc(&d_data, max_total);
    if (e == cudaSuccess) e = m.alloc(&d_s2l, 256);
    if (e == cudaSuccess) e = m.alloc(&d_thr, 255);
    if (e == cudaSuccess) e = cudaMemcpy(d_s2l, s2l_host, sizeof(s2l_host), cudaMemcpyHostToDevice);
    if (e == cudaSuccess) e = cudaMemcpy(d_thr, thr_host, sizeof(thr_host), cudaMemcpyHostToDevice);
    for (HTexture* t : textures) {
        if (e != cudaSuccess) break;
        if (t->max_mip == 0) continue;
        const uint32_t slices = t->type == SWR_TEX_CUBEMAP ? 6u : 1u;
        const size_t level0 = (size_t)t->width * t->height * slices;
        const size_t total =
            (size_t)t->mip_offsets[t->max_mip] + (size_t)t->mip_widths[t->max_mip] * t->mip_heights[t->max_mip] * slices;
        e = cudaMemcpy(d_data, t->data.data(), level0 * sizeof(uint32_t), cudaMemcpyHostToDevice);
        for (uint32_t mip = 1; mip <= t->max_mip && e == cudaSuccess; ++mip) {
            MipJob j;
            j.src = d_data + t->mip_offsets[mip - 1];
            j.dst = d_data + t->mip_offsets[mip];
            j.pw = t->mip_widths[mip - 1];
            j.ph = t->mip_heights[mip - 1];
            j.pstride = t->array_stride[mip - 1];
            j.mw = t->mip_widths[mip];
            j.mh = t->mip_heights[mip];
            j.slices = slices;
            j.type = t->type;
            k_mip<<<grid_for((uint64_t)j.mw * j.mh * slices, 256), 256>>>(j, d_s2l, d_thr);
            e = cudaGetLastError();
        }
        if (e != cudaSuccess) break;
        t->data.resize(total);
        e = cudaMemcpy(t->data.data(), d_data, total * sizeof(uint32_t), cudaMemcpyDeviceToHost);
    }
    if (e != cudaSuccess) return cuda_status(e, "device mip chains", err);
    return SWR_OK;
}

swr_status brdf_lut_device(uint32_t size, HTexture& out, std::string& err) {
    const uint32_t kSamples = 128;
    std::vector<float> xi_x(kSamples), xi_y(kSamples), c(kSamples), s(kSamples);
    hammersley_table(kSamples, xi_x.data(), xi_y.data(), c.data(), s.data());
    std::vector<float> samp(4 * kSamples);
    for (uint32_t i = 0; i < kSamples; ++i) {
        samp[4 * i] = xi_x[i];
        samp[4 * i + 1] = xi_y[i];
        samp[4 * i + 2] = c[i];
        samp[4 * i + 3] = s[i];
    }
    const size_t n = (size_t)size * size;
    out = HTexture{};
    out.width = out.height = size;
    out.type = SWR_TEX_LINEAR;
    out.data.resize(n);
    out.mip_offsets = {0};
    out.mip_widths = {size};
    out.mip_heights = {size};
    out.mip_widths_f = {(float)size};
    out.mip_heights_f = {(float)size};
    out.array_stride = {0};
    out.whv[0] = out.whv[1] = out.whv[2] = out.whv[3] = (float)size;
    {
        Mem m;
        float4* d_samp = nullptr;
        uint32_t* d_out = nullptr;
        cudaError_t e = m.alloc(&d_samp, kSamples);
        if (e == cudaSuccess) e = m.alloc(&d_out, n);
        if (e == cudaSuccess) e = cudaMemcpy(d_samp, samp.data(), samp.size() * sizeof(float), cudaMemcpyHostToDevice);
        if (e == cudaSuccess) {
            k_brdf<<<grid_for(n, 128), 128>>>(size, d_samp, d_out);
            e = cudaGetLastError();
        }
        if (e == cudaSuccess) e = cudaMemcpy(out.data.data(), d_out, n * sizeof(uint32_t), cudaMemcpyDeviceToHost);
        if (e != cudaSuccess) return cuda_status(e, "device BRDF LUT", err);
    }
    return mipmaps_device({&out}, err);
}

swr_status prefiltered_specular_device(const HTexture& cube, uint32_t samples, HTexture& out, uint64_t& host_texels,
                                       std::string& err) {
    out = prefiltered_layout(cube.width, cube.height);
    std::vector<float> xi_x(samples), xi_y(samples), c(samples), s(samples);
    hammersley_table(samples, xi_x.data(), xi_y.data(), c.data(), s.data());
    std::vector<float> samp(4 * (size_t)samples);
    for (uint32_t i = 0; i < samples; ++i) {
        samp[4 * i] = xi_x[i];
        samp[4 * i + 1] = xi_y[i];
        samp[4 * i + 2] = c[i];
        samp[4 * i + 3] = s[i];
    }
    const size_t face = (size_t)cube.width * cube.height;
    const size_t n = out.data.size();
    if (n > 0xFFFFFFFFull) {
        // Texel indices are 32-bit (six 16384^2 faces of 15 mips would need more).
        err = "prefiltered environment too large";
        return SWR_INVALID_ARG;
    }
    Mem m;
    uint32_t *d_cube = nullptr, *d_out = nullptr, *d_flags = nullptr, *d_nflags = nullptr;
    float4* d_samp = nullptr;
    cudaError_t e = m.alloc(&d_cube, 6 * face);
    if (e == cudaSuccess) e = m.alloc(&d_out, n);
    if (e == cudaSuccess) e = m.alloc(&d_flags, n);
    if (e == cudaSuccess) e = m.alloc(&d_nflags, 1);
    if (e == cudaSuccess) e = m.alloc(&d_samp, std::max<uint32_t>(samples, 1));
    if (e == cudaSuccess) e = cudaMemcpy(d_cube, cube.data.data(), 6 * face * sizeof(uint32_t), cudaMemcpyHostToDevice);
    if (e == cudaSuccess && samples)
        e = cudaMemcpy(d_samp, samp.data(), samp.size() * sizeof(float), cudaMemcpyHostToDevice);
    if (e == cudaSuccess) e = cudaMemset(d_nflags, 0, sizeof(uint32_t));
    if (e == cudaSuccess) {
        PrefilterArgs a;
        a.cube = Cube{d_cube, cube.width, cube.height};
        a.max_mip = out.max_mip;
        a.samples = samples;
        a.samp = d_samp;
        a.out = d_out;
        a.flags = d_flags;
        a.nflags = d_nflags;
        k_prefilter<<<grid_for(n, 128), 128>>>(a);
        e = cudaGetLastError();
    }
    uint32_t nf = 0;
    if (e == cudaSuccess) e = cudaMemcpy(out.data.data(), d_out, n * sizeof(uint32_t), cudaMemcpyDeviceToHost);
    if (e == cudaSuccess) e = cudaMemcpy(&nf, d_nflags, sizeof(uint32_t), cudaMemcpyDeviceToHost);
    std::vector<uint32_t> flags(nf);
    if (e == cudaSuccess && nf) e = cudaMemcpy(flags.data(), d_flags, nf * sizeof(uint32_t), cudaMemcpyDeviceToHost);
    if (e != cudaSuccess) return cuda_status(e, "device GGX prefilter", err);
    for (uint32_t idx : flags) {
        const uint32_t mip = (uint32_t)(idx / (6 * face));
        const uint32_t rem = (uint32_t)(idx - (size_t)mip * 6 * face);
        const uint32_t f = (uint32_t)(rem / face);
        const uint32_t t = (uint32_t)(rem - f * face);
        const uint32_t y = t / cube.width, x = t - y * cube.width;
        out.data[idx] = prefilter_texel(cube, mip, out.max_mip, f, x, y, samples, xi_x.data(), xi_y.data());
    }
    host_texels += nf;
    return SWR_OK;
}

swr_status srgb_pow_selftest(const float* in, float* out, uint64_t n, uint32_t mode, std::string& err) {
    if (n == 0) return SWR_OK;
    Mem m;
    float *d_in = nullptr, *d_out = nullptr;
    cudaError_t e = m.alloc(&d_in, n);
    if (e == cudaSuccess) e = m.alloc(&d_out, n);
    if (e == cudaSuccess) e = cudaMemcpy(d_in, in, n * sizeof(float), cudaMemcpyHostToDevice);
    if (e == cudaSuccess) {
        k_pow_selftest<<<grid_for(n, 256), 256>>>(d_in, d_out, n, mode);
        e = cudaGetLastError();
    }
    if (e == cudaSuccess) e = cudaMemcpy(out, d_out, n * sizeof(float), cudaMemcpyDeviceToHost);
    if (e != cudaSuccess) return cuda_status(e, "powf self-test", err);
    return SWR_OK;
}

}  // namespace swr
