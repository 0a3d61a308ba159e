// cvshim_prims.cpp -- ORACLE / TEST INFRASTRUCTURE ONLY.
// Restatements of the OpenCV 3.2 primitives used by ORB-SLAM2's front-end;
// the definitions each one follows are listed in cvshim_prims.h.
#include "cvshim_prims.h"

#include <cmath>
#include <cstdlib>
#include <cstring>
#include <vector>

extern "C" {

int shim_cvround_f(float v) { return (int)std::lrint(v); }
int shim_cvround_d(double v) { return (int)std::lrint(v); }

static inline int shim_floor_f(float v) {
    int i = (int)v;
    return i - (i > v);
}

int shim_border_reflect101(int p, int len) {
    if (len == 1) return 0;
    while (p < 0 || p >= len) {
        if (p < 0) p = -p;
        else p = 2 * len - 2 - p;
    }
    return p;
}

static inline short sat_short_round(float v) {
    int r = shim_cvround_f(v);
    if (r < -32768) r = -32768;
    if (r > 32767) r = 32767;
    return (short)r;
}

static inline uint8_t sat_u8(int v) { return (uint8_t)(v < 0 ? 0 : (v > 255 ? 255 : v)); }

// cv::resize, INTER_LINEAR, 8-bit: coefficients are saturate_cast<short>(w * 2048)
// of the float weights (1-f, f) at source position (d + 0.5) * scale - 0.5;
// the horizontal pass keeps 2048-scaled ints, the vertical pass combines two
// of them with the 2048-scaled row weights and rounds with (v + 2^21) >> 22.
void shim_resize_linear_u8(const uint8_t* src, size_t sstep, int sw, int sh,
                           uint8_t* dst, size_t dstep, int dw, int dh) {
    const double inv_scale_x = (double)dw / sw, inv_scale_y = (double)dh / sh;
    const double scale_x = 1. / inv_scale_x, scale_y = 1. / inv_scale_y;
    std::vector<int> xofs(dw);
    std::vector<short> alpha(2 * dw);
    int xmax = dw;
    for (int dx = 0; dx < dw; dx++) {
        float fx = (float)((dx + 0.5) * scale_x - 0.5);
        int sx = shim_floor_f(fx);
        fx -= sx;
        if (sx < 0) { fx = 0.f; sx = 0; }
        if (sx + 1 >= sw) {
            if (dx < xmax) xmax = dx;
            if (sx >= sw - 1) { fx = 0.f; sx = sw - 1; }
        }
        xofs[dx] = sx;
        alpha[2 * dx] = sat_short_round((1.f - fx) * 2048);
        alpha[2 * dx + 1] = sat_short_round(fx * 2048);
    }
    std::vector<int> h0(dw), h1(dw);
    auto hrow = [&](int sy, std::vector<int>& h) {
        const uint8_t* S = src + (size_t)sy * sstep;
        int dx = 0;
        for (; dx < xmax; dx++) {
            int sx = xofs[dx];
            h[dx] = S[sx] * alpha[2 * dx] + S[sx + 1] * alpha[2 * dx + 1];
        }
        for (; dx < dw; dx++) h[dx] = S[xofs[dx]] * 2048;
    };
    for (int dy = 0; dy < dh; dy++) {
        float fy = (float)((dy + 0.5) * scale_y - 0.5);
        int sy = shim_floor_f(fy);
        fy -= sy;
        const int b0 = sat_short_round((1.f - fy) * 2048);
        const int b1 = sat_short_round(fy * 2048);
        int r0 = sy < 0 ? 0 : (sy >= sh ? sh - 1 : sy);
        int r1 = sy + 1 < 0 ? 0 : (sy + 1 >= sh ? sh - 1 : sy + 1);
        hrow(r0, h0);
        hrow(r1, h1);
        uint8_t* D = dst + (size_t)dy * dstep;
        for (int dx = 0; dx < dw; dx++) D[dx] = sat_u8((h0[dx] * b0 + h1[dx] * b1 + (1 << 21)) >> 22);
    }
}

// getGaussianKernel(7, 2, CV_32F) converted to CV_32S with scale 256.
void shim_gauss7_taps(int taps[7]) {
    const int n = 7;
    const double sigma = 2.0;
    const double scale2X = -0.5 / (sigma * sigma);
    float cf[7];
    double sum = 0;
    for (int i = 0; i < n; i++) {
        double x = i - (n - 1) * 0.5;
        double t = std::exp(scale2X * x * x);
        cf[i] = (float)t;
        sum += cf[i];
    }
    sum = 1. / sum;
    for (int i = 0; i < n; i++) cf[i] = (float)(cf[i] * sum);
    for (int i = 0; i < n; i++) taps[i] = shim_cvround_f(cf[i] * 256.f);
}

void shim_gauss7_u8(const uint8_t* src, size_t sstep, int w, int h, uint8_t* dst, size_t dstep) {
    int k[7];
    shim_gauss7_taps(k);
    std::vector<int> rows((size_t)w * h);
    for (int y = 0; y < h; y++) {
        const uint8_t* S = src + (size_t)y * sstep;
        for (int x = 0; x < w; x++) {
            int s = 0;
            for (int j = -3; j <= 3; j++) s += k[j + 3] * S[shim_border_reflect101(x + j, w)];
            rows[(size_t)y * w + x] = s;
        }
    }
    for (int y = 0; y < h; y++) {
        uint8_t* D = dst + (size_t)y * dstep;
        for (int x = 0; x < w; x++) {
            int s = 0;
            for (int j = -3; j <= 3; j++) s += k[j + 3] * rows[(size_t)shim_border_reflect101(y + j, h) * w + x];
            D[x] = sat_u8((s + (1 << 15)) >> 16);
        }
    }
}

// Bresenham circle of radius 3, in cyclic order around the centre.
static const int kCircle[16][2] = {{0, 3},  {1, 3},   {2, 2},   {3, 1},   {3, 0},  {3, -1},
                                   {2, -2}, {1, -3},  {0, -3},  {-1, -3}, {-2, -2}, {-3, -1},
                                   {-3, 0}, {-3, 1},  {-2, 2},  {-1, 3}};

int shim_fast_arc_strength(const uint8_t* c, size_t step) {
    int d[16];
    const int v = c[0];
    for (int k = 0; k < 16; k++) d[k] = v - c[kCircle[k][0] + (ptrdiff_t)kCircle[k][1] * (ptrdiff_t)step];
    int best = 0;
    for (int k = 0; k < 16; k++) {
        int mn_pos = 1 << 30, mn_neg = 1 << 30;
        for (int j = 0; j < 9; j++) {
            int e = d[(k + j) & 15];
            if (e < mn_pos) mn_pos = e;
            if (-e < mn_neg) mn_neg = -e;
        }
        if (mn_pos > best) best = mn_pos;
        if (mn_neg > best) best = mn_neg;
    }
    return best;
}

int shim_fast9_u8(const uint8_t* img, size_t step, int w, int h, int threshold, shim_corner* out, int cap) {
    if (threshold < 0) threshold = 0;
    if (threshold > 255) threshold = 255;
    int n = 0;
    if (w < 7 || h < 7) return 0;
    // score map: corner score where the segment test passes, 0 elsewhere
    // (non-corners and the 3-pixel frame count as 0 in the suppression).
    std::vector<int> score((size_t)w * h, 0);
    std::vector<uint8_t> corner((size_t)w * h, 0);
    for (int y = 3; y < h - 3; y++)
        for (int x = 3; x < w - 3; x++) {
            int m = shim_fast_arc_strength(img + (size_t)y * step + x, step);
            if (m > threshold) {
                score[(size_t)y * w + x] = m - 1;
                corner[(size_t)y * w + x] = 1;
            }
        }
    for (int y = 3; y < h - 3; y++)
        for (int x = 3; x < w - 3; x++) {
            if (!corner[(size_t)y * w + x]) continue;
            const int s = score[(size_t)y * w + x];
            bool keep = true;
            for (int dy = -1; dy <= 1 && keep; dy++)
                for (int dx = -1; dx <= 1; dx++) {
                    if (!dx && !dy) continue;
                    if (!(s > score[(size_t)(y + dy) * w + (x + dx)])) { keep = false; break; }
                }
            if (keep) {
                if (n < cap) { out[n].x = x; out[n].y = y; out[n].score = s; }
                n++;
            }
        }
    return n;
}

// atan2 in degrees from a 7th-order odd minimax polynomial of atan on [0, 1].
static const float kAtanP1 = 0.9997878412794807f * (float)(180 / 3.141592653589793238);
static const float kAtanP3 = -0.3258083974640975f * (float)(180 / 3.141592653589793238);
static const float kAtanP5 = 0.1555786518463281f * (float)(180 / 3.141592653589793238);
static const float kAtanP7 = -0.04432655554792128f * (float)(180 / 3.141592653589793238);

float shim_fast_atan2(float y, float x) {
    float ax = std::fabs(x), ay = std::fabs(y);
    float a, c, c2;
    const float eps = (float)2.220446049250313e-16;
    if (ax >= ay) {
        c = ay / (ax + eps);
        c2 = c * c;
        a = (((kAtanP7 * c2 + kAtanP5) * c2 + kAtanP3) * c2 + kAtanP1) * c;
    } else {
        c = ax / (ay + eps);
        c2 = c * c;
        a = 90.f - (((kAtanP7 * c2 + kAtanP5) * c2 + kAtanP3) * c2 + kAtanP1) * c;
    }
    if (x < 0) a = 180.f - a;
    if (y < 0) a = 360.f - a;
    return a;
}

}  // extern "C"
