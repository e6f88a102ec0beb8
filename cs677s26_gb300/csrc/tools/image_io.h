// Host image helpers of the command-line drop-ins: binary PGM in, PPM out,
// and the crop-resize of mined windows (src/main.cu:245-371).
#pragma once

#include <algorithm>
#include <cctype>
#include <cmath>
#include <cstdint>
#include <cstdio>
#include <fstream>
#include <iostream>
#include <string>
#include <vector>

#include "vjgb.h"

namespace vjtools {

struct Gray {
    int w = 0, h = 0;
    std::vector<uint8_t> px;
};

// Whole-file read in 1 MiB pieces.  0: ok, 1: cannot open, 2: read error.
inline int read_file(const std::string& path, std::vector<uint8_t>& bytes) {
    bytes.clear();
    std::FILE* fp = std::fopen(path.c_str(), "rb");
    if (!fp) return 1;
    constexpr size_t kPiece = 1u << 20;
    size_t got = 0;
    for (;;) {
        bytes.resize(got + kPiece);
        const size_t r = std::fread(bytes.data() + got, 1, kPiece, fp);
        got += r;
        if (r < kPiece) break;
    }
    const bool bad = std::ferror(fp) != 0;
    std::fclose(fp);
    bytes.resize(got);
    return bad ? 2 : 0;
}

// Netpbm P5 header reader over a byte buffer: fields are separated by
// whitespace, and a '#' starts a comment that runs to the end of its line.
struct PnmHeader {
    const std::vector<uint8_t>& b;
    size_t at = 0;
    static bool space(uint8_t c) { return c == ' ' || c == '\t' || c == '\n' || c == '\r' || c == '\v' || c == '\f'; }
    void skip() {
        while (at < b.size()) {
            if (b[at] == '#') {
                while (at < b.size() && b[at] != '\n') ++at;
            } else if (space(b[at])) {
                ++at;
            } else {
                break;
            }
        }
    }
    // A decimal field; false when it is missing, not a number or above 2^30.
    bool number(int& v) {
        skip();
        int64_t acc = 0;
        const size_t from = at;
        while (at < b.size() && b[at] >= '0' && b[at] <= '9') {
            acc = acc * 10 + (b[at++] - '0');
            if (acc > (1 << 30)) return false;
        }
        if (at == from) return false;
        v = static_cast<int>(acc);
        return true;
    }
};

// Binary P5 PGM with maxval <= 255 (the reference's loadPGM, main.cu:315-354,
// accepts the same files and prints the same messages).
inline bool load_pgm(const std::string& path, Gray& g, bool quiet = false) {
    std::vector<uint8_t> bytes;
    if (read_file(path, bytes) == 1) {
        if (!quiet) std::cerr << "[ERR] Cannot open PGM: " << path << "\n";
        return false;
    }
    PnmHeader hdr{bytes};
    hdr.skip();
    const bool magic = hdr.at + 2 <= bytes.size() && bytes[hdr.at] == 'P' && bytes[hdr.at + 1] == '5' &&
                       (hdr.at + 2 == bytes.size() || PnmHeader::space(bytes[hdr.at + 2]) || bytes[hdr.at + 2] == '#');
    if (!magic) {
        if (!quiet) std::cerr << "[ERR] Unsupported PGM format (need P5): " << path << "\n";
        return false;
    }
    hdr.at += 2;
    int w = 0, h = 0, maxVal = 0;
    if (!hdr.number(w) || !hdr.number(h) || !hdr.number(maxVal) || w <= 0 || h <= 0 || maxVal <= 0 ||
        maxVal > 255) {
        if (!quiet) std::cerr << "[ERR] Invalid PGM metadata\n";
        return false;
    }
    // exactly one whitespace byte separates the header from the raster
    const size_t raster = hdr.at + 1;
    const size_t need = static_cast<size_t>(w) * static_cast<size_t>(h);
    if (raster > bytes.size() || bytes.size() - raster < need) {
        if (!quiet) std::cerr << "[ERR] Failed to read PGM pixel payload\n";
        return false;
    }
    g.w = w;
    g.h = h;
    g.px.assign(bytes.begin() + static_cast<std::ptrdiff_t>(raster),
                bytes.begin() + static_cast<std::ptrdiff_t>(raster + need));
    return true;
}

inline bool save_ppm(const std::string& path, int w, int h, const std::vector<uint8_t>& rgb) {
    std::ofstream ofs(path, std::ios::binary);
    if (!ofs) {
        std::cerr << "[ERR] Cannot write PPM: " << path << "\n";
        return false;
    }
    ofs << "P6\n" << w << " " << h << "\n255\n";
    ofs.write(reinterpret_cast<const char*>(rgb.data()), static_cast<std::streamsize>(rgb.size()));
    return static_cast<bool>(ofs);
}

// 2-pixel white frame, clipped to the image (drawRect, main.cu:373-409).
inline void draw_frame(std::vector<uint8_t>& rgb, int w, int h, const vj_detection& d) {
    const int x0 = std::max(0, d.x), y0 = std::max(0, d.y);
    const int x1 = std::min(w - 1, d.x + d.w - 1), y1 = std::min(h - 1, d.y + d.h - 1);
    if (x0 > x1 || y0 > y1) return;
    auto set = [&](int x, int y) {
        const size_t i = (static_cast<size_t>(y) * w + x) * 3;
        rgb[i] = rgb[i + 1] = rgb[i + 2] = 255;
    };
    for (int t = 0; t < 2; ++t) {
        const int yt = std::min(h - 1, y0 + t), yb = std::max(0, y1 - t);
        for (int x = x0; x <= x1; ++x) {
            set(x, yt);
            set(x, yb);
        }
        const int xl = std::min(w - 1, x0 + t), xr = std::max(0, x1 - t);
        for (int y = y0; y <= y1; ++y) {
            set(xl, y);
            set(xr, y);
        }
    }
}

// The window (x, y, w, h) of `img` resized to out x out with pixel-centre
// bilinear sampling and round-half-up (cropResizeTo24, main.cu:245-284).
inline void crop_resize(const Gray& img, int x, int y, int w, int h, int out, uint8_t* dst) {
    const float sx = static_cast<float>(std::max(1, w));
    const float sy = static_cast<float>(std::max(1, h));
    for (int oy = 0; oy < out; ++oy) {
        for (int ox = 0; ox < out; ++ox) {
            const float fx = static_cast<float>(x) + (static_cast<float>(ox) + 0.5f) * (sx / out) - 0.5f;
            const float fy = static_cast<float>(y) + (static_cast<float>(oy) + 0.5f) * (sy / out) - 0.5f;
            const int x0 = std::clamp(static_cast<int>(std::floor(fx)), 0, img.w - 1);
            const int y0 = std::clamp(static_cast<int>(std::floor(fy)), 0, img.h - 1);
            const int x1 = std::min(x0 + 1, img.w - 1);
            const int y1 = std::min(y0 + 1, img.h - 1);
            const float ax = fx - static_cast<float>(x0);
            const float ay = fy - static_cast<float>(y0);
            const float p00 = img.px[static_cast<size_t>(y0) * img.w + x0];
            const float p01 = img.px[static_cast<size_t>(y0) * img.w + x1];
            const float p10 = img.px[static_cast<size_t>(y1) * img.w + x0];
            const float p11 = img.px[static_cast<size_t>(y1) * img.w + x1];
            const float top = p00 + (p01 - p00) * ax;
            const float bot = p10 + (p11 - p10) * ax;
            const float val = top + (bot - top) * ay;
            dst[static_cast<size_t>(oy) * out + ox] = static_cast<uint8_t>(std::clamp(static_cast<int>(val + 0.5f), 0, 255));
        }
    }
}

}  // namespace vjtools
