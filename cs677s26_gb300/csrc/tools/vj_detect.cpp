// vj_detect: the drop-in for `cuda_hello detect` (src/main.cu:2394-2579).
//
//   vj_detect <in_model.bin> <image.pgm> <out.ppm>
//             [scaleFactor=1.25] [minNeighbors=4] [minObjectSize=24]
//             [maxDetections=200000] [benchmarkRuns=0]
//
// Same arguments, defaults and clamps, same console lines, same output image:
// the grey input as RGB with a 2-pixel white frame around every grouped
// detection, written as binary PPM.  Detection runs through the library's
// C ABI (vj_detect with grouping), i.e. the GB300 kernels.
#include <algorithm>
#include <cctype>
#include <chrono>
#include <cstdint>
#include <cstdio>
#include <fstream>
#include <iostream>
#include <limits>
#include <string>
#include <vector>

#include <cuda_runtime.h>

#include "image_io.h"
#include "vjgb.h"

namespace {

using vjtools::Gray;
using vjtools::draw_frame;
using vjtools::load_pgm;
using vjtools::save_ppm;

int fail(const char* what) {
    std::cerr << "[ERR] " << what << " failed: " << vj_last_error() << "\n";
    return 1;
}

}  // namespace

int main(int argc, char** argv) {
    if (argc < 4) {
        std::cerr << "Usage: vj_detect <in_model.bin> <image.pgm> <out.ppm>"
                  << " [scaleFactor=1.25] [minNeighbors=4] [minObjectSize=24] [maxDetections=200000] "
                     "[benchmarkRuns=0]\n";
        return 1;
    }
    const std::string modelPath = argv[1], imagePath = argv[2], outPath = argv[3];
    float scaleFactor = 1.25f;
    int minNeighbors = 4, minObjectSize = 24, maxDetections = 200000, benchmarkRuns = 0;
    try {
        if (argc > 4) scaleFactor = std::stof(argv[4]);
        if (argc > 5) minNeighbors = std::max(1, std::stoi(argv[5]));
        if (argc > 6) minObjectSize = std::max(1, std::stoi(argv[6]));
        if (argc > 7) maxDetections = std::max(100, std::stoi(argv[7]));
        if (argc > 8) benchmarkRuns = std::max(0, std::stoi(argv[8]));
    } catch (...) {
        std::cerr << "[ERR] Invalid numeric argument\n";
        return 1;
    }

    int winW = 0, winH = 0;
    int64_t nf = 0, ns = 0, nst = 0;
    if (vj_model_load_header(modelPath.c_str(), &winW, &winH, &nf, &ns, &nst) != VJ_OK) {
        std::cerr << "[ERR] loadCascadeModel failed: " << modelPath << " (" << vj_last_error() << ")\n";
        return 1;
    }
    std::vector<vj_haar_feature> feats(static_cast<size_t>(nf));
    std::vector<vj_stump4> stumps(static_cast<size_t>(ns));
    std::vector<vj_cascade_stage> stages(static_cast<size_t>(nst));
    if (vj_model_load(modelPath.c_str(), feats.data(), nf, stumps.data(), ns, stages.data(), nst) != VJ_OK) {
        std::cerr << "[ERR] loadCascadeModel failed: " << modelPath << " (" << vj_last_error() << ")\n";
        return 1;
    }
    Gray img;
    if (!load_pgm(imagePath, img)) return 1;

    vj_detector* det = nullptr;
    if (vj_detector_create(winW, winH, std::max(winW, img.w), std::max(winH, img.h), maxDetections, &det) != VJ_OK)
        return fail("detector create");
    if (vj_detector_set_model(det, feats.data(), nf, stumps.data(), ns, stages.data(), nst) != VJ_OK)
        return fail("setCascadeModel");
    // The reference uploads the image once and detects from device memory.
    uint8_t* dImage = nullptr;
    if (cudaMalloc(&dImage, img.px.size()) != cudaSuccess ||
        cudaMemcpy(dImage, img.px.data(), img.px.size(), cudaMemcpyHostToDevice) != cudaSuccess) {
        std::cerr << "[ERR] cudaMemcpy to device failed\n";
        return 1;
    }
    std::vector<vj_detection> dets(static_cast<size_t>(maxDetections));
    int count = 0;
    auto detect = [&]() {
        return vj_detect(det, dImage, img.w, img.h, img.w, 1, scaleFactor, minNeighbors, minObjectSize, maxDetections,
                         1, dets.data(), maxDetections, &count, nullptr);
    };
    if (benchmarkRuns > 0) {
        for (int i = 0; i < 3; ++i)
            if (detect() != VJ_OK) return fail("warmup detectMultiScale");
        double sum = 0.0, mn = std::numeric_limits<double>::infinity(), mx = 0.0;
        for (int i = 0; i < benchmarkRuns; ++i) {
            const auto t0 = std::chrono::steady_clock::now();
            if (detect() != VJ_OK) return fail("detectMultiScale");
            const double ms = std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - t0).count();
            sum += ms;
            mn = std::min(mn, ms);
            mx = std::max(mx, ms);
        }
        const double avg = sum / benchmarkRuns;
        std::cout << "[DETECT_BENCH] runs=" << benchmarkRuns << " detections(last)=" << count << " avg(ms): " << avg
                  << " min(ms): " << mn << " max(ms): " << mx << " avg(fps): " << (avg > 0.0 ? 1000.0 / avg : 0.0)
                  << "\n";
    } else {
        const auto t0 = std::chrono::high_resolution_clock::now();
        if (detect() != VJ_OK) return fail("detectMultiScale");
        const auto ms =
            std::chrono::duration_cast<std::chrono::milliseconds>(std::chrono::high_resolution_clock::now() - t0)
                .count();
        std::cout << "[DETECT] detections=" << count << " elapsed(ms): " << ms << "\n";
    }
    std::vector<uint8_t> rgb(static_cast<size_t>(img.w) * img.h * 3);
    for (size_t i = 0; i < img.px.size(); ++i) rgb[3 * i] = rgb[3 * i + 1] = rgb[3 * i + 2] = img.px[i];
    for (int i = 0; i < count; ++i) draw_frame(rgb, img.w, img.h, dets[static_cast<size_t>(i)]);
    cudaFree(dImage);
    vj_detector_destroy(det);
    if (!save_ppm(outPath, img.w, img.h, rgb)) {
        std::cerr << "[ERR] savePPM failed\n";
        return 1;
    }
    std::cout << "[OK] Saved result to: " << outPath << "\n";
    return 0;
}
