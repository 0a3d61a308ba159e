// orbgpu_sincos.cu -- host construction of the descriptor-angle sin/cos
// exception table.
//
// computeOrbDescriptor (src/ORBextractor.cc:156-157) rotates the test pattern
// by a = (float)cos(angle), b = (float)sin(angle) with angle a float in
// [0, 2*pi], i.e. by the host C library's cosf/sinf.  The device evaluates
// sincos_taylor (IEEE double arithmetic only, identical on host and device)
// and rounds to float; this file lists, for every float input in range, the
// ones where that rounding differs from the host library, so the device can
// return the library's value for them.  The list is built once per machine
// (at build time) and cached next to the library.
#include <dlfcn.h>
#include <gnu/libc-version.h>
#include <sys/utsname.h>

#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <string>
#include <thread>
#include <vector>

#include "orbgpu_host.h"

namespace orbgpu {

// The table belongs to one C library build: its name carries the machine
// and the glibc version.
std::string default_sincos_table_path() {
    struct utsname u;
    std::string tag = "unknown";
    if (uname(&u) == 0) tag = u.machine;
    tag += std::string("_glibc") + gnu_get_libc_version();
    const std::string name = "sincos_exceptions_" + tag + ".bin";
    Dl_info info;
    if (dladdr((void*)&default_sincos_table_path, &info) && info.dli_fname) {
        std::string p(info.dli_fname);
        const size_t s = p.find_last_of('/');
        if (s != std::string::npos) return p.substr(0, s + 1) + name;
    }
    return name;
}

static inline uint32_t fbits(float f) {
    uint32_t u;
    std::memcpy(&u, &f, 4);
    return u;
}
static inline float bitsf(uint32_t u) {
    float f;
    std::memcpy(&f, &u, 4);
    return f;
}

int build_sincos_table(const char* path, int threads) {
    const float factorPI = (float)(3.1415926535897932384626433832795 / 180.f);
    volatile float deg = 360.f;
    const float hi = deg * factorPI;
    const uint32_t n = fbits(hi) + 1;  // every float in [0, hi]
    if (threads < 1) threads = 1;
    struct Part {
        std::vector<uint32_t> ck, sk;
        std::vector<float> cv, sv;
    };
    std::vector<Part> parts(threads);
    std::vector<std::thread> pool;
    for (int t = 0; t < threads; t++)
        pool.emplace_back([&, t]() {
            const uint32_t lo = (uint32_t)((uint64_t)n * t / threads), up = (uint32_t)((uint64_t)n * (t + 1) / threads);
            Part& P = parts[t];
            for (uint32_t u = lo; u < up; u++) {
                const float x = bitsf(u);
                double sd, cd;
                sincos_taylor(x, &sd, &cd);
                const float c0 = (float)cd, s0 = (float)sd;
                const float c1 = cosf(x), s1 = sinf(x);
                if (fbits(c0) != fbits(c1)) {
                    P.ck.push_back(u);
                    P.cv.push_back(c1);
                }
                if (fbits(s0) != fbits(s1)) {
                    P.sk.push_back(u);
                    P.sv.push_back(s1);
                }
            }
        });
    for (auto& th : pool) th.join();
    std::vector<uint32_t> ck, sk;
    std::vector<float> cv, sv;
    for (auto& P : parts) {
        ck.insert(ck.end(), P.ck.begin(), P.ck.end());
        cv.insert(cv.end(), P.cv.begin(), P.cv.end());
        sk.insert(sk.end(), P.sk.begin(), P.sk.end());
        sv.insert(sv.end(), P.sv.begin(), P.sv.end());
    }
    FILE* f = std::fopen(path, "wb");
    if (!f) return ORBGPU_ERR_BAD_ARG;
    const int32_t hdr[4] = {0x4f524258, (int32_t)ck.size(), (int32_t)sk.size(), 0};
    std::fwrite(hdr, sizeof(int32_t), 4, f);
    std::fwrite(ck.data(), 4, ck.size(), f);
    std::fwrite(cv.data(), 4, cv.size(), f);
    std::fwrite(sk.data(), 4, sk.size(), f);
    std::fwrite(sv.data(), 4, sv.size(), f);
    std::fclose(f);
    return ORBGPU_OK;
}

}  // namespace orbgpu

// Builds the exception table (see above); 'path' NULL = next to the library.
extern "C" int orbgpu_build_sincos_table(const char* path, int threads) {
    std::string p = path ? path : orbgpu::default_sincos_table_path();
    return orbgpu::build_sincos_table(p.c_str(), threads);
}

extern "C" const char* orbgpu_sincos_table_path(void) {
    static std::string p = orbgpu::default_sincos_table_path();
    return p.c_str();
}

