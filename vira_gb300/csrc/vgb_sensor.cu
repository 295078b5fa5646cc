// vgb_sensor.cu -- the sensor chain after the film and the PSF convolution.
//
// k_sensor restates Camera::simulateSensor (cameras/camera.ipp:1218-1240) per pixel:
// getPhotonCounts (camera.ipp:1286-1330), NoiseModel::simulate with its fixed pattern
// (noise_models/noise_model.ipp:36-74) and Photosite::exposePixel (photosites/photosite.ipp:
// 125-136), in the reference's FP32 operation order.  Random draws come from Philox-4x32-10
// keyed by (seed, frame) with the counter (pixel, purpose, frame, 0xE0): exact Poisson samples by
// inversion below a mean of 10 and by Hormann's transformed rejection (PTRS, 1993) above,
// Gaussian samples by Box-Muller.
//
// k_psf restates Image::convolveSpatial (images/image.ipp:1267-1340): a correlation with a
// centred kernel and zero padding, kernel rows outer, each output summed in the reference's
// order; an output tile and its halo are staged in shared memory.
#include <cuda_runtime.h>

#include <algorithm>
#include <cstdint>

#include "vgb_device.cuh"
#include "vgb_internal.h"

using namespace vgbd;

namespace {

constexpr uint32_t kSlotSensor = 0xE0u;

__device__ __forceinline__ float u01_open(uint32_t x) {  // (0, 1]
    return ((float)(x >> 8) + 1.0f) * (1.0f / 16777216.0f);
}

// -lambda + k ln(lambda) - ln(k!), the log of the Poisson pmf up to its normalisation, formed
// without the cancellation of its large terms: for k >= 10 with Stirling's series for ln(k!)
// (z = k + 1: (z - 1/2) ln z - z + ln(2 pi)/2 + 1/(12 z) - 1/(360 z^3)), rearranged as
// k ln(lambda / z) + (z - lambda) - ln(z)/2 - ln(2 pi)/2 - 1/(12 z) + 1/(360 z^3); below 10 with
// exact ln(k!).
__device__ __forceinline__ float log_pmf_ratio(float lambda, float loglam, float kf) {
    if (kf < 10.f) {
        const float lnfact[10] = {0.f, 0.f, 0.6931472f, 1.7917595f, 3.1780539f,
                                  4.7874917f, 6.5792512f, 8.5251614f, 10.6046029f, 12.8018275f};
        return -lambda + kf * loglam - lnfact[(int)kf];
    }
    const float z = kf + 1.f;
    const float iz = 1.f / z;
    return kf * log1pf((lambda - z) * iz) + (z - lambda) - 0.5f * logf(z) - 0.91893853f - iz * (1.f / 12.f) +
           iz * iz * iz * (1.f / 360.f);
}

// Poisson(lambda) for lambda >= 0: inversion (sequential search) below 10, PTRS above.  Both
// loops are bounded; the rejection loop accepts with probability ~0.9 per round, and after 64
// rounds (never expected) returns the rounded mean.  Out of line: one copy serves every band.
__device__ __noinline__ float poisson(float lambda, uint32_t c0, uint32_t c1, uint32_t c2, uint32_t k0, uint32_t k1) {
    if (!(lambda > 0.f)) return 0.f;
    if (lambda < 10.f) {
        const U4 r = philox(U4{c0, c1, c2, kSlotSensor}, k0, k1);
        const float u = u01(r.x);
        float p = expf(-lambda), F = p;
        int k = 0;
        while (u > F && k < 1000) {
            ++k;
            p *= lambda / (float)k;
            F += p;
        }
        return (float)k;
    }
    const float slam = sqrtf(lambda), loglam = logf(lambda);
    const float b = 0.931f + 2.53f * slam;
    const float a = -0.059f + 0.02483f * b;
    const float invalpha = 1.1239f + 1.1328f / (b - 3.4f);
    const float vr = 0.9277f - 3.6224f / (b - 2.f);
    for (uint32_t round = 0; round < 64; ++round) {
        const U4 r = philox(U4{c0, c1 + (round << 16), c2, kSlotSensor | 1u}, k0, k1);
        const float U = u01(r.x) - 0.5f, V = u01_open(r.y);
        const float us = 0.5f - fabsf(U);
        const float kf = floorf((2.f * a / us + b) * U + lambda + 0.43f);
        if (us >= 0.07f && V <= vr) return kf;
        if (kf < 0.f || (us < 0.013f && V > us)) continue;
        if (logf(V) + logf(invalpha) - logf(a / (us * us) + b) <= log_pmf_ratio(lambda, loglam, kf)) return kf;
    }
    return rintf(lambda);
}

__device__ __forceinline__ float gaussian(float mean, float std, uint32_t c0, uint32_t c1, uint32_t c2, uint32_t k0,
                                          uint32_t k1) {
    const U4 r = philox(U4{c0, c1, c2, kSlotSensor | 2u}, k0, k1);
    const float u1 = u01_open(r.x), u2 = u01(r.y);
    return mean + std * (sqrtf(-2.f * logf(u1)) * cosf(6.2831853f * u2));
}

template <int NB>
__global__ void k_sensor(const float* __restrict__ power, uint32_t W, uint32_t H, uint32_t nb,
                         const vgb::SensorParams sp, float* __restrict__ image) {
    const size_t P = (size_t)W * H;
    const uint32_t k0 = (uint32_t)sp.seed, k1 = (uint32_t)(sp.seed >> 32);
    for (size_t p = (size_t)blockIdx.x * blockDim.x + threadIdx.x; p < P; p += (size_t)gridDim.x * blockDim.x) {
        const uint32_t i = (uint32_t)(p % W), j = (uint32_t)(p / W);
        float ph[NB];
        float total = 0.f;
#pragma unroll
        for (int k = 0; k < NB; ++k) {
            ph[k] = 0.f;
            if (k >= (int)nb) continue;
            float e = sp.exposure_time * power[k * P + p];
            if (sp.mosaic) e = e * sp.mosaic[k * P + p];
            ph[k] = e / sp.photon_energy[k];
            total += ph[k];
        }
        if (sp.photon_noise && total >= 1.f) {
#pragma unroll
            for (int k = 0; k < NB; ++k)
                if (k < (int)nb) ph[k] = poisson(ph[k], (uint32_t)p, (uint32_t)k, sp.frame, k0, k1);
        }
        float noise = 0.f;
        if (sp.noise_model) {
            const float dark = poisson(sp.dark_current, (uint32_t)p, 0x100u, sp.frame, k0, k1) * sp.exposure_time;
            const float readout = gaussian(sp.readout_mean, sp.readout_std, (uint32_t)p, 0x101u, sp.frame, k0, k1);
            float scale = 1.f;
            if (sp.hperiod != 0)
                scale *= (1.f - sp.hscale) +
                         (sp.hscale * (1.f + sinf(2.f * kPi * (float)i / (2.f * (float)sp.hperiod))));
            if (sp.vperiod != 0)
                scale *= (1.f - sp.vscale) +
                         (sp.vscale * (1.f + sinf(2.f * kPi * (float)j / (2.f * (float)sp.vperiod))));
            noise = scale * (dark + readout);
        }
        float electrons = 0.f;
#pragma unroll
        for (int k = 0; k < NB; ++k)
            if (k < (int)nb) electrons += sp.quantum_efficiency[k] * ph[k];
        electrons = electrons + noise;
        const float amplified = smin(sp.gain * electrons, sp.max_adu);
        image[p] = amplified / sp.max_adu;
    }
}

// NoiseModel::simulate (noise_models/noise_model.ipp:36-74) for one draw: dark-current Poisson
// counts times the exposure plus Gaussian readout, scaled by the sinusoidal fixed pattern.
// `purpose` separates the draws of one pixel (the RGB sensor draws once per channel).
__device__ __forceinline__ float noise_draw(const vgb::SensorParams& sp, uint32_t p, uint32_t i, uint32_t j,
                                            uint32_t purpose, uint32_t k0, uint32_t k1) {
    const float dark = poisson(sp.dark_current, p, purpose, sp.frame, k0, k1) * sp.exposure_time;
    const float readout = gaussian(sp.readout_mean, sp.readout_std, p, purpose + 1u, sp.frame, k0, k1);
    float scale = 1.f;
    if (sp.hperiod != 0)
        scale *= (1.f - sp.hscale) + (sp.hscale * (1.f + sinf(2.f * kPi * (float)i / (2.f * (float)sp.hperiod))));
    if (sp.vperiod != 0)
        scale *= (1.f - sp.vscale) + (sp.vscale * (1.f + sinf(2.f * kPi * (float)j / (2.f * (float)sp.vperiod))));
    return scale * (dark + readout);
}

// Camera::simulateSensorRGB per pixel (camera.ipp:1253-1282, 1337-1380; photosite.ipp:145-154),
// FP32 in the reference's order; spectralConvert's integrateOver (spectral_data.ipp:306-333) per
// RGB band.  Random draws: photon noise at purpose 0x200 + channel, the noise model's at
// 0x110 + 0x10 * channel (and + 1).
template <int NB>
__global__ void k_sensor_rgb(const float* __restrict__ power, uint32_t W, uint32_t H, uint32_t nb,
                             const vgb::SensorParams sp, const vgb::RgbParams rp, float* __restrict__ out) {
    const size_t P = (size_t)W * H;
    const uint32_t k0 = (uint32_t)sp.seed, k1 = (uint32_t)(sp.seed >> 32);
    for (size_t p = (size_t)blockIdx.x * blockDim.x + threadIdx.x; p < P; p += (size_t)gridDim.x * blockDim.x) {
        const uint32_t i = (uint32_t)(p % W), j = (uint32_t)(p / W);
        float v[NB];
#pragma unroll
        for (int k = 0; k < NB; ++k) {
            v[k] = 0.f;
            if (k < (int)nb) v[k] = sp.mosaic ? power[k * P + p] * sp.mosaic[k * P + p] : power[k * P + p];
        }
        float ph[3];
        float total = 0.f;
#pragma unroll
        for (int c = 0; c < 3; ++c) {
            const float lo = rp.rgb_min[c], hi = rp.rgb_max[c];
            float integral = 0.f;
#pragma unroll
            for (int k = 0; k < NB; ++k) {
                if (k >= (int)nb) break;
                const float bmin = rp.band_min[k], bmax = rp.band_max[k];
                if (bmin > hi || bmax < lo) continue;
                const float b1 = smax(bmin, lo), b2 = smin(bmax, hi);
                integral += (b2 - b1) * v[k];
            }
            const float rgb = integral / rp.rgb_bw[c];
            ph[c] = (sp.exposure_time * rgb) / rp.rgb_pe[c];
            total += ph[c];
        }
        if (sp.photon_noise && total >= 1.f) {
#pragma unroll
            for (int c = 0; c < 3; ++c) ph[c] = poisson(ph[c], (uint32_t)p, 0x200u + c, sp.frame, k0, k1);
        }
#pragma unroll
        for (int c = 0; c < 3; ++c) {
            const float noise = sp.noise_model ? noise_draw(sp, (uint32_t)p, i, j, 0x110u + 0x10u * c, k0, k1) : 0.f;
            const float electrons = (rp.rgb_qe[c] * ph[c]) + noise;
            out[c * P + p] = (sp.gain * electrons) / sp.max_adu;
        }
    }
}

constexpr int kTileW = 128, kTileH = 8;  // outputs per block: 32 threads x 4 columns, 8 rows
constexpr int kMaxKernel = 127;

__host__ __device__ constexpr int round4(int v) { return (v + 3) & ~3; }

// One block: a 128x8 output tile of one band.  Each thread owns 4 adjacent outputs of a row;
// the input tile (with its halo) and the band's kernel (rows padded to a multiple of 4 with
// zeros, never summed) sit in dynamic shared memory, read as float4: per 4 kernel taps a
// thread loads one float4 of input and one of kernel for 16 multiply-adds.  Every output is
// summed over ky outer, kx inner, as the reference's loop.
__global__ void __launch_bounds__(256) k_psf(const float* __restrict__ in, float* __restrict__ out, uint32_t W,
                                             uint32_t H, const float* __restrict__ kernel, int kw, int kh) {
    extern __shared__ float4 sm4[];
    float* sm = reinterpret_cast<float*>(sm4);
    const int band = blockIdx.z;
    const size_t P = (size_t)W * H;
    const float* src = in + band * P;
    const float* ker = kernel + (size_t)band * kw * kh;
    const int hw = kw / 2, hh = kh / 2;
    const int kwp = round4(kw);
    const int tw = round4(kTileW + kwp + 3), th = kTileH + kh - 1;
    float* tile = sm;
    float* ks = sm + (size_t)tw * th;
    const int x0 = blockIdx.x * kTileW - hw, y0 = blockIdx.y * kTileH - hh;
    const int tid = threadIdx.y * 32 + threadIdx.x, nthr = 32 * kTileH;
    for (int q = tid; q < tw * th; q += nthr) {
        const int ix = x0 + q % tw, iy = y0 + q / tw;
        tile[q] = (ix >= 0 && ix < (int)W && iy >= 0 && iy < (int)H) ? src[(size_t)iy * W + ix] : 0.f;
    }
    for (int q = tid; q < kwp * kh; q += nthr) {
        const int kx = q % kwp, ky = q / kwp;
        ks[q] = kx < kw ? ker[ky * kw + kx] : 0.f;
    }
    __syncthreads();
    const int xo = blockIdx.x * kTileW + 4 * threadIdx.x, y = blockIdx.y * kTileH + threadIdx.y;
    if (y >= (int)H || xo >= (int)W) return;
    float s0 = 0.f, s1 = 0.f, s2 = 0.f, s3 = 0.f;
    for (int ky = 0; ky < kh; ++ky) {
        const float4* row = reinterpret_cast<const float4*>(tile + (threadIdx.y + ky) * tw + 4 * threadIdx.x);
        const float4* krow = reinterpret_cast<const float4*>(ks + ky * kwp);
        float4 a = row[0];
        for (int c = 0; c < kwp / 4; ++c) {
            const float4 b = row[c + 1];
            const float4 k = krow[c];
            const float in[8] = {a.x, a.y, a.z, a.w, b.x, b.y, b.z, b.w};
            const float kk[4] = {k.x, k.y, k.z, k.w};
#pragma unroll
            for (int t = 0; t < 4; ++t) {
                if (4 * c + t >= kw) break;  // padded taps are not summed
                s0 += in[t] * kk[t];
                s1 += in[t + 1] * kk[t];
                s2 += in[t + 2] * kk[t];
                s3 += in[t + 3] * kk[t];
            }
            a = b;
        }
    }
    float* o = out + band * P + (size_t)y * W + xo;
    o[0] = s0;
    if (xo + 1 < (int)W) o[1] = s1;
    if (xo + 2 < (int)W) o[2] = s2;
    if (xo + 3 < (int)W) o[3] = s3;
}

}  // namespace

namespace vgb {

int launch_sensor(void* stream, const float* power, uint32_t width, uint32_t height, uint32_t nbands,
                  const SensorParams& sp, float* image, int num_sms) {
    const size_t P = (size_t)width * height;
    const int g = (int)std::max<size_t>(1, std::min<size_t>((P + 255) / 256, (size_t)num_sms * 8));
    cudaStream_t s = (cudaStream_t)stream;
    if (nbands <= 1) k_sensor<1><<<g, 256, 0, s>>>(power, width, height, nbands, sp, image);
    else if (nbands <= 4) k_sensor<4><<<g, 256, 0, s>>>(power, width, height, nbands, sp, image);
    else k_sensor<8><<<g, 256, 0, s>>>(power, width, height, nbands, sp, image);
    return (int)cudaGetLastError();
}

int launch_sensor_rgb(void* stream, const float* power, uint32_t width, uint32_t height, uint32_t nbands,
                      const SensorParams& sp, const RgbParams& rp, float* image_rgb, int num_sms) {
    const size_t P = (size_t)width * height;
    const int g = (int)std::max<size_t>(1, std::min<size_t>((P + 255) / 256, (size_t)num_sms * 8));
    cudaStream_t s = (cudaStream_t)stream;
    if (nbands <= 1) k_sensor_rgb<1><<<g, 256, 0, s>>>(power, width, height, nbands, sp, rp, image_rgb);
    else if (nbands <= 4) k_sensor_rgb<4><<<g, 256, 0, s>>>(power, width, height, nbands, sp, rp, image_rgb);
    else k_sensor_rgb<8><<<g, 256, 0, s>>>(power, width, height, nbands, sp, rp, image_rgb);
    return (int)cudaGetLastError();
}

int launch_psf(void* stream, const float* in, float* out, uint32_t width, uint32_t height, uint32_t nbands,
               const float* kernel, uint32_t kw, uint32_t kh) {
    if (kw > (uint32_t)kMaxKernel || kh > (uint32_t)kMaxKernel) return (int)cudaErrorInvalidValue;
    const int kwp = round4((int)kw);
    const size_t tw = round4(kTileW + kwp + 3), th = kTileH + kh - 1;
    const size_t smem = (tw * th + (size_t)kwp * kh) * sizeof(float);
    cudaError_t e = cudaFuncSetAttribute(k_psf, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e != cudaSuccess) return (int)e;
    const dim3 grid((width + kTileW - 1) / kTileW, (height + kTileH - 1) / kTileH, nbands);
    k_psf<<<grid, dim3(32, kTileH), smem, (cudaStream_t)stream>>>(in, out, width, height, kernel, (int)kw, (int)kh);
    return (int)cudaGetLastError();
}

}  // namespace vgb
