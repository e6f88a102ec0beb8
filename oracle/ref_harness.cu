// ref_harness.cu - exposes the reference's own CPU functions through a C ABI
// so the oracle can be checked against them.  TEST INFRASTRUCTURE: built by
// oracle/Makefile from the reference sources where they lie (REF=...), into
// oracle/_ref/ (git-ignored).  Nothing here is copied from the reference: the
// reference's src/main.cu is #included with its `main` renamed, and the
// functions below only marshal arguments into the reference's CPU paths:
//   buildHaarFeaturePool   face_vision_engine.cu:882-1020
//   buildHostIntegralImage main.cu:428-474
//   runCpuWeakSearch       main.cu:587-682
//   resizeGrayBilinearHost main.cu:545-585
//   detectMultiScaleCpu    main.cu:684-827
//   groupRectanglesCpu     face_vision_engine.cu:1401-1539
//   ModelIO save/load      model_io.cpp:66-167
//   cropResizeTo24         main.cu:245-284
#include <algorithm>
#include <array>
#include <chrono>
#include <climits>
#include <cmath>
#include <cstdint>
#include <cstdlib>
#include <cstring>
#include <filesystem>
#include <fstream>
#include <iostream>
#include <limits>
#include <numeric>
#include <random>
#include <sstream>
#include <string>
#include <vector>
#include <cuda_runtime.h>
#include <cub/cub.cuh>

// groupRectanglesCpu is a private member; open the class for this TU only.
#define private public
#include "vj/face_vision_engine.cuh"
#undef private

#define main reference_main
#include "../src/main.cu"
#undef main

extern "C" {

long long ref_pool(int mode, vj::HaarFeature* out, long long cap) {
    const auto pool = vj::FaceVisionEngine::buildHaarFeaturePool(
        vj::WindowSpec{24, 24}, static_cast<vj::FaceVisionEngine::FeatureMode>(mode));
    const long long n = static_cast<long long>(pool.size());
    if (out) std::memcpy(out, pool.data(), sizeof(vj::HaarFeature) * static_cast<size_t>(std::min(n, cap)));
    return n;
}

// Integral image of one w x h image, int32 sum/sqsum (h+1)x(w+1) and invNorm.
void ref_integral(const uint8_t* gray, int w, int h, int stride, int32_t* sum, int32_t* sq,
                  float* invNorm) {
    const HostIntegralImage ii = buildHostIntegralImage(gray, w, h, stride, true);
    std::memcpy(sum, ii.sum.data(), ii.sum.size() * sizeof(int32_t));
    std::memcpy(sq, ii.sqsum.data(), ii.sqsum.size() * sizeof(int32_t));
    *invNorm = ii.invNorm;
}

// runCpuWeakSearch over `features` (nFeat entries; the caller passes a masked
// subset when a used mask applies), n 24x24 patches.
void ref_weak_search(const vj::HaarFeature* features, int nFeat, const uint8_t* patches, int n,
                     const int8_t* labels, const uint8_t* active, const float* weights,
                     int* featureIdx, float* err, float* theta, int* parity) {
    std::vector<vj::HaarFeature> f(features, features + nFeat);
    std::vector<HostIntegralImage> s;
    s.reserve(static_cast<size_t>(n));
    for (int i = 0; i < n; ++i) s.push_back(buildHostIntegralImage(patches + static_cast<size_t>(i) * 576, 24, 24, 24, true));
    std::vector<int8_t> l(labels, labels + n);
    std::vector<uint8_t> a;
    if (active) a.assign(active, active + n);
    std::vector<float> w(weights, weights + n);
    const CpuBestWeakResult r = runCpuWeakSearch(f, nFeat, s, l, a, w);
    *featureIdx = r.featureIdx;
    *err = r.err;
    *theta = r.theta;
    *parity = r.parity;
}

void ref_resize(const uint8_t* src, int sw, int sh, int ss, uint8_t* dst, int dw, int dh) {
    const auto v = resizeGrayBilinearHost(src, sw, sh, ss, dw, dh);
    std::memcpy(dst, v.data(), v.size());
}

int ref_detect(const vj::HaarFeature* feats, int nFeat, const vj::GpuStump4* stumps, int nStumps,
               const vj::CascadeStage* stages, int nStages, const uint8_t* image, int w, int h,
               int stride, float sf, int minObj, int maxDet, int maxScales, vj::Detection* out,
               int cap) {
    std::vector<vj::HaarFeature> f(feats, feats + nFeat);
    std::vector<vj::GpuStump4> s(stumps, stumps + nStumps);
    std::vector<vj::CascadeStage> st(stages, stages + nStages);
    const auto d = detectMultiScaleCpu(f, s, st, vj::WindowSpec{24, 24}, image, w, h, stride, sf, minObj,
                                       maxDet, maxScales);
    const int k = std::min(static_cast<int>(d.size()), cap);
    std::memcpy(out, d.data(), sizeof(vj::Detection) * static_cast<size_t>(k));
    return static_cast<int>(d.size());
}

// groupRectanglesCpu does not read any member; it is called on raw storage
// because constructing an engine would allocate device memory.
int ref_group(const vj::Detection* in, int n, int minNeighbors, float eps, vj::Detection* out, int cap) {
    alignas(vj::FaceVisionEngine) static unsigned char storage[sizeof(vj::FaceVisionEngine)];
    const auto* eng = reinterpret_cast<const vj::FaceVisionEngine*>(storage);
    std::vector<vj::Detection> v(in, in + n);
    const auto g = eng->groupRectanglesCpu(v, minNeighbors, eps);
    const int k = std::min(static_cast<int>(g.size()), cap);
    std::memcpy(out, g.data(), sizeof(vj::Detection) * static_cast<size_t>(k));
    return static_cast<int>(g.size());
}

int ref_model_save(const char* path, const vj::HaarFeature* f, long long nf, const vj::GpuStump4* s,
                   long long ns, const vj::CascadeStage* st, long long nst) {
    std::vector<vj::HaarFeature> vf(f, f + nf);
    std::vector<vj::GpuStump4> vs(s, s + ns);
    std::vector<vj::CascadeStage> vst(st, st + nst);
    return vj::ModelIO::saveCascadeModel(path, vj::WindowSpec{24, 24}, vf, vs, vst) ? 1 : 0;
}

// cropResizeTo24 of the window (x, y, bw, bh) of a w x h image (no row padding).
void ref_crop(const uint8_t* img, int w, int h, int x, int y, int bw, int bh, uint8_t* out24) {
    GrayImage g;
    g.w = w;
    g.h = h;
    g.data.assign(img, img + static_cast<size_t>(w) * h);
    vj::Detection d{};
    d.x = x;
    d.y = y;
    d.w = bw;
    d.h = bh;
    std::vector<uint8_t> o;
    cropResizeTo24(g, d, o);
    std::memcpy(out24, o.data(), o.size());
}

}  // extern "C"
