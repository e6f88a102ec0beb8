// cropResizeTo24 (src/main.cu:245-284) on the device: the hard-negative
// miner's crop of each detected window, resized to the training window with
// pixel-centre bilinear interpolation, for many windows of many device images
// in one launch.  Every operation is one IEEE single rounding in the
// reference's order (explicit __fadd_rn / __fmul_rn, a correctly rounded
// division), so the patches equal the reference CPU function byte for byte.
#include <algorithm>
#include <string>
#include <vector>

#include "device_util.cuh"

namespace vjgb {
namespace {

struct CropJob {
    const uint8_t* img;
    int64_t stride;
    int w, h;
    int x, y;
    float stepX, stepY;  // max(1, bw) / out, max(1, bh) / out
};

__global__ void __launch_bounds__(256) crop_resize_kernel(const CropJob* __restrict__ jobs, int64_t total, int out,
                                                          uint8_t* __restrict__ dst) {
    const int64_t per = static_cast<int64_t>(out) * out;
    for (int64_t t = static_cast<int64_t>(blockIdx.x) * blockDim.x + threadIdx.x; t < total;
         t += static_cast<int64_t>(gridDim.x) * blockDim.x) {
        const int64_t k = t / per;
        const int r = static_cast<int>(t - k * per);
        const int oy = r / out, ox = r - oy * out;
        const CropJob J = jobs[k];
        const float fx = __fsub_rn(
            __fadd_rn(static_cast<float>(J.x), __fmul_rn(__fadd_rn(static_cast<float>(ox), 0.5f), J.stepX)), 0.5f);
        const float fy = __fsub_rn(
            __fadd_rn(static_cast<float>(J.y), __fmul_rn(__fadd_rn(static_cast<float>(oy), 0.5f), J.stepY)), 0.5f);
        const int x0 = min(max(static_cast<int>(floorf(fx)), 0), J.w - 1);
        const int y0 = min(max(static_cast<int>(floorf(fy)), 0), J.h - 1);
        const int x1 = min(x0 + 1, J.w - 1);
        const int y1 = min(y0 + 1, J.h - 1);
        const float ax = __fsub_rn(fx, static_cast<float>(x0));
        const float ay = __fsub_rn(fy, static_cast<float>(y0));
        const uint8_t* r0 = J.img + static_cast<int64_t>(y0) * J.stride;
        const uint8_t* r1 = J.img + static_cast<int64_t>(y1) * J.stride;
        const float p00 = static_cast<float>(r0[x0]), p01 = static_cast<float>(r0[x1]);
        const float p10 = static_cast<float>(r1[x0]), p11 = static_cast<float>(r1[x1]);
        const float top = __fadd_rn(p00, __fmul_rn(__fsub_rn(p01, p00), ax));
        const float bot = __fadd_rn(p10, __fmul_rn(__fsub_rn(p11, p10), ax));
        const float val = __fadd_rn(top, __fmul_rn(__fsub_rn(bot, top), ay));
        const int v = __float2int_rz(__fadd_rn(val, 0.5f));
        dst[t] = static_cast<uint8_t>(v < 0 ? 0 : (v > 255 ? 255 : v));
    }
}

}  // namespace
}  // namespace vjgb

using namespace vjgb;

extern "C" {

int vj_crop_resize_batch(int nImages, const uint8_t* const* images, const int* w, const int* h, const int* stride,
                         int nCrops, const int* imageOf, const vj_detection* boxes, int outSize, uint8_t* d_out,
                         void* stream) {
    if (nImages < 1 || !images || !w || !h || !stride || nCrops < 0 || outSize < 1 || outSize > 1024 ||
        (nCrops > 0 && (!imageOf || !boxes || !d_out)))
        return set_error(VJ_INVALID_ARG, "vj_crop_resize_batch: bad arguments");
    for (int i = 0; i < nImages; ++i)
        if (!images[i] || w[i] <= 0 || h[i] <= 0 || stride[i] < w[i])
            return set_error(VJ_INVALID_ARG, "vj_crop_resize_batch: bad image " + std::to_string(i));
    if (nCrops == 0) return ok();
    std::vector<CropJob> jobs(static_cast<size_t>(nCrops));
    for (int k = 0; k < nCrops; ++k) {
        const int i = imageOf[k];
        if (i < 0 || i >= nImages) return set_error(VJ_INVALID_ARG, "vj_crop_resize_batch: bad image index");
        CropJob& J = jobs[static_cast<size_t>(k)];
        J.img = images[i];
        J.stride = stride[i];
        J.w = w[i];
        J.h = h[i];
        J.x = boxes[k].x;
        J.y = boxes[k].y;
        // the reference divides max(1, w) by the int window size in float
        J.stepX = static_cast<float>(boxes[k].w > 1 ? boxes[k].w : 1) / static_cast<float>(outSize);
        J.stepY = static_cast<float>(boxes[k].h > 1 ? boxes[k].h : 1) / static_cast<float>(outSize);
    }
    const cudaStream_t s = static_cast<cudaStream_t>(stream);
    CropJob* dj = nullptr;
    VJ_CUDA_TRY(cudaMallocAsync(reinterpret_cast<void**>(&dj), sizeof(CropJob) * jobs.size(), s));
    cudaError_t e = cudaMemcpyAsync(dj, jobs.data(), sizeof(CropJob) * jobs.size(), cudaMemcpyHostToDevice, s);
    const int64_t total = static_cast<int64_t>(nCrops) * outSize * outSize;
    if (e == cudaSuccess) {
        int dev = 0, sms = 0;
        cudaGetDevice(&dev);
        cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
        // grid-stride loop: at most 16 blocks of 256 threads per SM of this device
        const int64_t blocks = std::min<int64_t>((total + 255) / 256, int64_t(sms > 0 ? sms : 1) * 16);
        crop_resize_kernel<<<static_cast<unsigned>(blocks), 256, 0, s>>>(dj, total, outSize, d_out);
        e = cudaGetLastError();
    }
    const cudaError_t f = cudaFreeAsync(dj, s);
    if (e != cudaSuccess) return set_error(VJ_CUDA_ERROR, std::string("vj_crop_resize_batch: ") + cudaGetErrorString(e));
    if (f != cudaSuccess) return set_error(VJ_CUDA_ERROR, std::string("vj_crop_resize_batch: ") + cudaGetErrorString(f));
    return ok();
}

}  // extern "C"
