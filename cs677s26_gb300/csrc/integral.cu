// Integral and squared-integral images on sm_103a.
//
// Reference: RowPrefixKernel + ColumnScanTransposeKernel /
// ColumnScanTransposeSingleSampleKernel + ComputeInvNormKernel
// (src/face_vision_engine.cu:47-259, driver :1057-1158).  The reference keeps
// int32 sums and int32 squared sums (wrapping mod 2^32); here sums are uint32
// (the same bits) and squared sums are exact uint64 whose low 32 bits are the
// reference's bits.
//
// Training batches (24x24 patches, transposed [625][n] layout): one thread
// per sample keeps its running column sums in registers and writes each
// integral pixel for 32 consecutive samples per warp store, so every store is
// a full 128-byte (sum) / 256-byte (squared sum) line.
//
// Detection levels (row-major): a row pass (one warp per row, 16 pixels per
// lane, warp shuffle scan, 16-byte stores of exclusive prefixes), then two
// column passes over 32-column x 32-row segments: segment totals, then the
// in-place column scan with the carry of the segments above.  All levels of
// all images of a batch go through one launch of each pass.
#include <cmath>
#include <mutex>
#include <string>
#include <vector>

#include <cuda.h>  // CUcontext / CUresult types only; the driver is reached through the runtime

#include "integral_dev.cuh"

namespace vjgb {
namespace {

// invNorm of face_vision_engine.cu:216-259: over the interior
// (1, 1, iiW-3, iiH-3), each corner read as the reference's int32 value and
// converted to double, nf2 = area*sq - s*s, 1/sqrt(nf2) rounded to float.
__device__ __forceinline__ float inv_norm(uint32_t s0, uint32_t s1, uint32_t s2, uint32_t s3, uint64_t q0,
                                          uint64_t q1, uint64_t q2, uint64_t q3, int iiW, int iiH) {
    if (iiW < 3 || iiH < 3) return 1.0f;
    const double area = static_cast<double>((iiW - 3) * (iiH - 3));
    auto i2d = [](uint32_t v) { return static_cast<double>(static_cast<int32_t>(v)); };
    auto q2d = [](uint64_t v) { return static_cast<double>(static_cast<int32_t>(static_cast<uint32_t>(v))); };
    const double s = i2d(s0) - i2d(s1) - i2d(s2) + i2d(s3);
    const double q = q2d(q0) - q2d(q1) - q2d(q2) + q2d(q3);
    const double nf2 = area * q - s * s;
    return nf2 > 1e-12 ? static_cast<float>(1.0 / sqrt(nf2)) : 0.0f;
}

// 24x24 training patches, one thread per sample.
__global__ void __launch_bounds__(128)
train_integral24_kernel(const uint8_t* __restrict__ gray, int stride, int n, uint32_t* __restrict__ sumT,
                        uint64_t* __restrict__ sqT, float* __restrict__ invNorm) {
    constexpr int W = 24, IIW = 25;
    const int s = blockIdx.x * blockDim.x + threadIdx.x;
    if (s >= n) return;
    const size_t N = static_cast<size_t>(n);
    const uint8_t* img = gray + static_cast<size_t>(s) * W * stride;
    uint32_t cs[W];
    uint64_t cq[W];
#pragma unroll
    for (int x = 0; x < W; ++x) {
        cs[x] = 0;
        cq[x] = 0;
    }
#pragma unroll
    for (int c = 0; c < IIW; ++c) {
        sumT[c * N + s] = 0;
        if (sqT) sqT[c * N + s] = 0;
    }
    uint32_t k11 = 0, k23 = 0, k1y = 0, k2y = 0;
    uint64_t q11 = 0, q23 = 0, q1y = 0, q2y = 0;
    for (int y = 1; y <= W; ++y) {
        const uint8_t* prow = img + static_cast<size_t>(y - 1) * stride;
        uint8_t px[W];
#pragma unroll
        for (int x = 0; x < W; ++x) px[x] = __ldg(prow + x);
        const size_t rb = static_cast<size_t>(y) * IIW;
        sumT[rb * N + s] = 0;
        if (sqT) sqT[rb * N + s] = 0;
        uint32_t rs = 0, rq = 0;
#pragma unroll
        for (int x = 0; x < W; ++x) {
            rs += px[x];
            rq += static_cast<uint32_t>(px[x]) * px[x];
            cs[x] += rs;
            cq[x] += rq;
            sumT[(rb + x + 1) * N + s] = cs[x];
            if (sqT) sqT[(rb + x + 1) * N + s] = cq[x];
        }
        if (y == 1) {
            k11 = cs[0];
            k23 = cs[22];
            q11 = cq[0];
            q23 = cq[22];
        }
        if (y == 23) {
            k1y = cs[0];
            k2y = cs[22];
            q1y = cq[0];
            q2y = cq[22];
        }
    }
    if (invNorm) invNorm[s] = inv_norm(k11, k23, k1y, k2y, q11, q23, q1y, q2y, IIW, IIW);
}

// Any patch size: same arithmetic, previous integral row read back.
__global__ void __launch_bounds__(128)
train_integral_generic_kernel(const uint8_t* __restrict__ gray, int w, int h, int stride, int n,
                              uint32_t* __restrict__ sumT, uint64_t* __restrict__ sqT, float* __restrict__ invNorm) {
    const int s = blockIdx.x * blockDim.x + threadIdx.x;
    if (s >= n) return;
    const size_t N = static_cast<size_t>(n);
    const int iiW = w + 1, iiH = h + 1;
    const uint8_t* img = gray + static_cast<size_t>(s) * h * stride;
    for (int c = 0; c < iiW; ++c) {
        sumT[c * N + s] = 0;
        if (sqT) sqT[c * N + s] = 0;
    }
    for (int y = 1; y <= h; ++y) {
        const uint8_t* prow = img + static_cast<size_t>(y - 1) * stride;
        const size_t rb = static_cast<size_t>(y) * iiW;
        sumT[rb * N + s] = 0;
        if (sqT) sqT[rb * N + s] = 0;
        uint32_t rs = 0;
        uint64_t rq = 0;
        for (int x = 1; x <= w; ++x) {
            const uint32_t p = prow[x - 1];
            rs += p;
            rq += p * p;
            const size_t i = rb + x;
            sumT[i * N + s] = sumT[(i - iiW) * N + s] + rs;
            if (sqT) sqT[i * N + s] = sqT[(i - iiW) * N + s] + rq;
        }
    }
    if (invNorm) {
        if (iiW < 3 || iiH < 3 || !sqT) {
            invNorm[s] = 1.0f;
            return;
        }
        const int ww = iiW - 3, hh = iiH - 3;
        const size_t p0 = 1 + iiW, p1 = (1 + ww) + iiW, p2 = 1 + static_cast<size_t>(iiW) * (1 + hh),
                     p3 = (1 + ww) + static_cast<size_t>(iiW) * (1 + hh);
        invNorm[s] = inv_norm(sumT[p0 * N + s], sumT[p1 * N + s], sumT[p2 * N + s], sumT[p3 * N + s],
                              sqT[p0 * N + s], sqT[p1 * N + s], sqT[p2 * N + s], sqT[p3 * N + s], iiW, iiH);
    }
}

// Row pass: one warp per integral row (integral_dev.cuh).
__global__ void __launch_bounds__(256)
row_pass_kernel(const IIJob* __restrict__ jobs, int njobs, int64_t rows) {
    const int lane = threadIdx.x & 31;
    const int64_t nw = (static_cast<int64_t>(gridDim.x) * blockDim.x) >> 5;
    for (int64_t r = (static_cast<int64_t>(blockIdx.x) * blockDim.x + threadIdx.x) >> 5; r < rows; r += nw)
        ii_row_item(jobs, njobs, r, lane);
}

// Column pass A: segment totals.
__global__ void __launch_bounds__(256)
col_total_kernel(const IIJob* __restrict__ jobs, int njobs, int64_t items, int64_t totPitch,
                 uint32_t* __restrict__ totS, uint64_t* __restrict__ totQ) {
    const int lane = threadIdx.x & 31;
    const int64_t nw = (static_cast<int64_t>(gridDim.x) * blockDim.x) >> 5;
    for (int64_t it = (static_cast<int64_t>(blockIdx.x) * blockDim.x + threadIdx.x) >> 5; it < items; it += nw)
        ii_col_total_item(jobs, njobs, it, lane, totPitch, totS, totQ);
}

// Column pass B: in-place column scan.
__global__ void __launch_bounds__(256)
col_scan_kernel(const IIJob* __restrict__ jobs, int njobs, int64_t items, int64_t totPitch,
                const uint32_t* __restrict__ totS, const uint64_t* __restrict__ totQ) {
    const int lane = threadIdx.x & 31;
    const int64_t nw = (static_cast<int64_t>(gridDim.x) * blockDim.x) >> 5;
    for (int64_t it = (static_cast<int64_t>(blockIdx.x) * blockDim.x + threadIdx.x) >> 5; it < items; it += nw)
        ii_col_scan_item(jobs, njobs, it, lane, totPitch, totS, totQ);
}

int grid_for(int64_t warps) {
    int dev = 0, sms = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    const int64_t blocks = (warps + 7) / 8;
    const int64_t cap = static_cast<int64_t>(sms > 0 ? sms : 1) * 16;
    return static_cast<int>(blocks < 1 ? 1 : (blocks < cap ? blocks : cap));
}

}  // namespace

int launch_integral_jobs(const IIJob* d_jobs, int njobs, const IIPlan& plan, uint32_t* d_totS, uint64_t* d_totQ,
                         cudaStream_t stream) {
    if (njobs <= 0) return VJ_OK;
    VJ_TIMED_LAUNCH("row_pass_kernel", stream,
                    row_pass_kernel<<<grid_for(plan.rows), 256, 0, stream>>>(d_jobs, njobs, plan.rows));
    VJ_LAUNCH_CHECK("row_pass_kernel");
    VJ_TIMED_LAUNCH("col_total_kernel", stream,
                    col_total_kernel<<<grid_for(plan.items), 256, 0, stream>>>(d_jobs, njobs, plan.items,
                                                                               plan.totPitch, d_totS, d_totQ));
    VJ_LAUNCH_CHECK("col_total_kernel");
    VJ_TIMED_LAUNCH("col_scan_kernel", stream,
                    col_scan_kernel<<<grid_for(plan.items), 256, 0, stream>>>(d_jobs, njobs, plan.items,
                                                                              plan.totPitch, d_totS, d_totQ));
    VJ_LAUNCH_CHECK("col_scan_kernel");
    return VJ_OK;
}

// ---------------------------------------------------------------------------
// Scratch of vj_integral_image_noalloc: a fixed array in device memory, sized
// for the largest image the variant accepts.
// ---------------------------------------------------------------------------
namespace {

constexpr int kNoAllocMaxW = 3840, kNoAllocMaxH = 2160;
constexpr int64_t kNoAllocTotRows = (kNoAllocMaxH + kColSeg - 1) / kColSeg;      // 68 segments
constexpr int64_t kNoAllocTotPitch = ((kNoAllocMaxW + 1 + 31) / 32) * 32;        // 3872 columns
constexpr size_t kNoAllocJobBytes = 256;
constexpr size_t kNoAllocTotS = static_cast<size_t>(kNoAllocTotRows * kNoAllocTotPitch) * sizeof(uint32_t);
constexpr size_t kNoAllocTotQ = static_cast<size_t>(kNoAllocTotRows * kNoAllocTotPitch) * sizeof(uint64_t);
constexpr size_t kNoAllocBytes = kNoAllocJobBytes + kNoAllocTotQ + kNoAllocTotS;
static_assert(sizeof(IIJob) <= kNoAllocJobBytes, "job descriptor fits its slot");

// Layout: [job descriptor | squared-sum totals | sum totals].
static __device__ __align__(256) unsigned char g_noalloc_scratch[kNoAllocBytes];

// The job descriptor travels as a kernel parameter, so no host buffer has to
// outlive the call.
__global__ void store_job_kernel(IIJob* dst, IIJob job) { *dst = job; }

constexpr int kMaxDevices = 64;
std::mutex g_noalloc_mu;
struct NoAllocSlot {
    unsigned long long ctx = 0;  // unique id of the context the address belongs to
    unsigned char* ptr = nullptr;
};
NoAllocSlot g_noalloc_slot[kMaxDevices];

// Unique id of the calling thread's current context, or 0 when it has none.
// cuCtxGetCurrent / cuCtxGetId are reached through the runtime's driver entry
// points, so the library does not link the driver library itself.
unsigned long long current_context_id() {
    using GetCurrent = CUresult (*)(CUcontext*);
    using GetId = CUresult (*)(CUcontext, unsigned long long*);
    static GetCurrent getCurrent = nullptr;
    static GetId getId = nullptr;
    static bool resolved = false;
    if (!resolved) {  // under g_noalloc_mu
        void* a = nullptr;
        void* b = nullptr;
        cudaDriverEntryPointQueryResult qa{}, qb{};
        if (cudaGetDriverEntryPointByVersion("cuCtxGetCurrent", &a, 12000, cudaEnableDefault, &qa) == cudaSuccess &&
            qa == cudaDriverEntryPointSuccess)
            getCurrent = reinterpret_cast<GetCurrent>(a);
        if (cudaGetDriverEntryPointByVersion("cuCtxGetId", &b, 12000, cudaEnableDefault, &qb) == cudaSuccess &&
            qb == cudaDriverEntryPointSuccess)
            getId = reinterpret_cast<GetId>(b);
        resolved = true;
    }
    CUcontext c = nullptr;
    unsigned long long id = 0;
    if (!getCurrent || !getId || getCurrent(&c) != CUDA_SUCCESS || !c || getId(c, &id) != CUDA_SUCCESS) return 0;
    return id;
}

// Device address of the scratch array in the current context.  The address
// belongs to the context that loaded the module: after cudaDeviceReset, or a
// primary context released and created again, the module loads again and the
// array may move.  So the address is cached per device together with the
// unique id of the context it was taken in, and looked up again (with that
// device current) whenever the current context differs.
int noalloc_scratch(unsigned char** out) {
    int dev = 0;
    VJ_CUDA_TRY(cudaGetDevice(&dev));
    if (dev < 0 || dev >= kMaxDevices) return set_error(VJ_RUNTIME_ERROR, "vj_integral_image_noalloc: device id");
    std::lock_guard<std::mutex> lk(g_noalloc_mu);
    NoAllocSlot& slot = g_noalloc_slot[dev];
    const unsigned long long ctx = current_context_id();
    if (!slot.ptr || ctx == 0 || slot.ctx != ctx) {
        void* p = nullptr;
        const cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
        if (e != cudaSuccess || !p)
            return set_error(VJ_CUDA_ERROR, std::string("vj_integral_image_noalloc: cudaGetSymbolAddress: ") +
                                                cudaGetErrorString(e));
        slot.ptr = static_cast<unsigned char*>(p);
        slot.ctx = current_context_id();  // the lookup creates the primary context if there was none
    }
    *out = slot.ptr;
    return VJ_OK;
}

}  // namespace
}  // namespace vjgb

using namespace vjgb;

extern "C" {

int vj_integral_image_noalloc(const uint8_t* d_gray, int w, int h, int stride, uint32_t* d_sum, uint64_t* d_sqsum,
                              void* stream) {
    if (!d_gray || !d_sum || !d_sqsum || w <= 0 || h <= 0 || stride < w)
        return set_error(VJ_INVALID_ARG, "vj_integral_image_noalloc: bad arguments (d_sqsum is required)");
    if (w > kNoAllocMaxW || h > kNoAllocMaxH)
        return set_error(VJ_INVALID_ARG, "vj_integral_image_noalloc: image larger than 3840 x 2160, the size its "
                                         "fixed scratch holds; use vj_integral_image");
    unsigned char* base = nullptr;
    const int st0 = noalloc_scratch(&base);
    if (st0 != VJ_OK) return st0;
    cudaStream_t s = static_cast<cudaStream_t>(stream);
    IIJob job{};
    job.pix = d_gray;
    job.stride = stride;
    job.sum = d_sum;
    job.sq = d_sqsum;
    job.w = w;
    job.h = h;
    job.pitch = w + 1;
    const IIPlan plan = plan_integral_jobs(&job, 1);
    IIJob* d_job = reinterpret_cast<IIJob*>(base);
    uint64_t* totQ = reinterpret_cast<uint64_t*>(base + kNoAllocJobBytes);
    uint32_t* totS = reinterpret_cast<uint32_t*>(base + kNoAllocJobBytes + kNoAllocTotQ);
    // Every total the column passes read is written first by col_total_kernel
    // in the same call, so nothing left by an earlier call is ever read.
    VJ_TIMED_LAUNCH("store_job_kernel", s, store_job_kernel<<<1, 1, 0, s>>>(d_job, job));
    VJ_LAUNCH_CHECK("store_job_kernel");
    const int st = launch_integral_jobs(d_job, 1, plan, totS, totQ, s);
    return st == VJ_OK ? ok() : st;
}

int vj_integral_batch(const uint8_t* d_gray, int w, int h, int stride, int n, uint32_t* d_sumT,
                      uint64_t* d_sqsumT, float* d_invNorm, void* stream) {
    if (!d_gray || !d_sumT || w <= 0 || h <= 0 || stride < w || n <= 0)
        return set_error(VJ_INVALID_ARG, "vj_integral_batch: bad arguments");
    if (static_cast<int64_t>(w) * h * 255 >= (1LL << 31))
        return set_error(VJ_INVALID_ARG, "vj_integral_batch: image too large for 32-bit sums");
    cudaStream_t s = static_cast<cudaStream_t>(stream);
    const int grid = div_up(n, 128);
    if (w == 24 && h == 24) {
        VJ_TIMED_LAUNCH("train_integral24_kernel", s,
                        train_integral24_kernel<<<grid, 128, 0, s>>>(d_gray, stride, n, d_sumT, d_sqsumT, d_invNorm));
    } else {
        if (d_invNorm && !d_sqsumT)
            return set_error(VJ_INVALID_ARG, "vj_integral_batch: invNorm needs the squared sums for this size");
        VJ_TIMED_LAUNCH("train_integral_generic_kernel", s,
                        train_integral_generic_kernel<<<grid, 128, 0, s>>>(d_gray, w, h, stride, n, d_sumT, d_sqsumT,
                                                                           d_invNorm));
    }
    VJ_LAUNCH_CHECK("train_integral_kernel");
    return ok();
}

int vj_integral_image(const uint8_t* d_gray, int w, int h, int stride, uint32_t* d_sum, uint64_t* d_sqsum,
                      void* stream) {
    if (!d_gray || !d_sum || w <= 0 || h <= 0 || stride < w || w > 65535 || h > 65535)
        return set_error(VJ_INVALID_ARG, "vj_integral_image: bad arguments");
    cudaStream_t s = static_cast<cudaStream_t>(stream);
    IIJob job{};
    job.pix = d_gray;
    job.stride = stride;
    job.sum = d_sum;
    job.w = w;
    job.h = h;
    job.pitch = w + 1;
    uint64_t* sq = d_sqsum;
    if (!sq) VJ_CUDA_TRY(cudaMallocAsync(reinterpret_cast<void**>(&sq), sizeof(uint64_t) * (w + 1) * (h + 1), s));
    job.sq = sq;
    IIPlan plan = plan_integral_jobs(&job, 1);
    IIJob* d_job = nullptr;
    uint32_t* totS = nullptr;
    uint64_t* totQ = nullptr;
    VJ_CUDA_TRY(cudaMallocAsync(reinterpret_cast<void**>(&d_job), sizeof(IIJob), s));
    VJ_CUDA_TRY(cudaMallocAsync(reinterpret_cast<void**>(&totS), sizeof(uint32_t) * plan.totRows * plan.totPitch, s));
    VJ_CUDA_TRY(cudaMallocAsync(reinterpret_cast<void**>(&totQ), sizeof(uint64_t) * plan.totRows * plan.totPitch, s));
    VJ_CUDA_TRY(cudaMemcpyAsync(d_job, &job, sizeof(IIJob), cudaMemcpyHostToDevice, s));
    const int st = launch_integral_jobs(d_job, 1, plan, totS, totQ, s);
    cudaFreeAsync(d_job, s);
    cudaFreeAsync(totS, s);
    cudaFreeAsync(totQ, s);
    if (!d_sqsum) cudaFreeAsync(sq, s);
    if (st != VJ_OK) return st;
    // The job descriptor lives on the host stack: finish the copy before returning.
    VJ_CUDA_TRY(cudaStreamSynchronize(s));
    return ok();
}

}  // extern "C"
