// orbgpu_match.cu -- the windowed descriptor searches and stereo matching.
//
// Distances and candidate windows are computed in parallel (one warp per
// query); the parts of the reference that are sequential by construction --
// a later query seeing the matches of earlier ones (vMatchedDistance in
// SearchForInitialization, claimed keypoints in SearchByProjection) -- are
// replayed in order by one warp over the precomputed candidate lists.
//
// Candidate order: Frame::GetFeaturesInArea (src/Frame.cc:590-670) visits
// grid cells column by column and each cell in keypoint-index order, so a
// candidate's position in that order is (cell x * 48 + cell y, index).  The
// searches compare candidates lexicographically on (distance, position),
// which reproduces the reference's "first strictly smaller wins" loops.
#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <vector>

#include "orbgpu_host.h"
#include "orbgpu_stereo.cuh"

namespace orbgpu {

#define PROJ_ROUNDS 12
#define PROJ_NONE 0x7f7f7f7f

struct GridDev {
    const orbgpu_keypoint* kps;
    const uint8_t* desc;
    const float* uright;
    int n;
    float minX, minY, invW, invH;
    const int* cell_start;  // 64*48 + 1
    const int* cell_keys;   // n
    const int* key_cell;    // n, -1 if outside the grid
    float scale[16];
};

// PosInGrid (src/Frame.cc:682-698).
__device__ __forceinline__ int pos_in_grid(const orbgpu_keypoint& kp, float minX, float minY, float invW, float invH) {
    const int px = (int)roundf(__fmul_rn(__fsub_rn(kp.x, minX), invW));
    const int py = (int)roundf(__fmul_rn(__fsub_rn(kp.y, minY), invH));
    if (px < 0 || px >= ORBGPU_GRID_COLS || py < 0 || py >= ORBGPU_GRID_ROWS) return -1;
    return px * ORBGPU_GRID_ROWS + py;
}

__global__ void k_grid_count(const orbgpu_keypoint* kps, int n, float minX, float minY, float invW, float invH,
                             int* key_cell, int* cell_count) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const int c = pos_in_grid(kps[i], minX, minY, invW, invH);
    key_cell[i] = c;
    if (c >= 0) atomicAdd(&cell_count[c], 1);
}

__global__ void k_grid_scan(const int* cell_count, int* cell_start, int* cursor) {
    __shared__ int s_scan[32];
    const int ncell = ORBGPU_GRID_COLS * ORBGPU_GRID_ROWS;
    int base = 0;
    for (int b0 = 0; b0 < ncell; b0 += blockDim.x) {
        const int c = b0 + threadIdx.x;
        const int v = c < ncell ? cell_count[c] : 0;
        int tot;
        const int ex = block_exclusive_scan(v, s_scan, &tot);
        if (c < ncell) {
            cell_start[c] = base + ex;
            cursor[c] = base + ex;
        }
        base += tot;
    }
    if (threadIdx.x == 0) cell_start[ncell] = base;
}

__global__ void k_grid_fill(const int* key_cell, int n, int* cursor, int* cell_keys) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const int c = key_cell[i];
    if (c >= 0) cell_keys[atomicAdd(&cursor[c], 1)] = i;
}

// Frame::GetFeaturesInArea cell range; false when the window misses the grid.
__device__ __forceinline__ bool area_cells(const GridDev& g, float x, float y, float r, int& x0, int& x1, int& y0,
                                           int& y1) {
    x0 = max(0, (int)floorf(__fmul_rn(__fsub_rn(__fsub_rn(x, g.minX), r), g.invW)));
    if (x0 >= ORBGPU_GRID_COLS) return false;
    x1 = min(ORBGPU_GRID_COLS - 1, (int)ceilf(__fmul_rn(__fadd_rn(__fsub_rn(x, g.minX), r), g.invW)));
    if (x1 < 0) return false;
    y0 = max(0, (int)floorf(__fmul_rn(__fsub_rn(__fsub_rn(y, g.minY), r), g.invH)));
    if (y0 >= ORBGPU_GRID_ROWS) return false;
    y1 = min(ORBGPU_GRID_ROWS - 1, (int)ceilf(__fmul_rn(__fadd_rn(__fsub_rn(y, g.minY), r), g.invH)));
    if (y1 < 0) return false;
    return true;
}

__device__ __forceinline__ bool in_area(const GridDev& g, int idx, float x, float y, float r, int minLevel,
                                        int maxLevel) {
    const orbgpu_keypoint kp = g.kps[idx];
    const bool check = (minLevel > 0) || (maxLevel >= 0);
    if (check) {
        if (kp.octave < minLevel) return false;
        if (maxLevel >= 0 && kp.octave > maxLevel) return false;
    }
    const float dx = __fsub_rn(kp.x, x), dy = __fsub_rn(kp.y, y);
    return __fadd_rn(__fmul_rn(dx, dx), __fmul_rn(dy, dy)) < __fmul_rn(r, r);
}

// Candidate record: distance, GetFeaturesInArea position, keypoint index, octave.
struct Cand {
    int dist;
    int idx;
    uint32_t order;  // cell << 16 | rank-free tie key: index
    int octave;
};

__device__ __forceinline__ uint64_t cand_key(int dist, int cell, int idx) {
    return ((uint64_t)(uint32_t)dist << 40) | ((uint64_t)(uint32_t)cell << 20) | (uint64_t)(uint32_t)idx;
}

// ----------------------------------------------------------------- SearchForInitialization
// Pass 1: count (fill == 0) or write (fill == 1) the candidates of every
// level-0 keypoint of F1 in the window around prev[i1] (src/ORBmatcher.cc:603-640).
__global__ void k_init_candidates(GridDev g2, const orbgpu_keypoint* kps1, const uint8_t* desc1, int n1,
                                  const float* prev, float window, const int* cand_start, int* cand_count,
                                  uint64_t* cand_out, int fill) {
    const int lane = threadIdx.x & 31;
    const int i1 = blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5);
    if (i1 >= n1) return;
    const orbgpu_keypoint kp1 = kps1[i1];
    int total = 0;
    int x0, x1, y0, y1;
    if (kp1.octave <= 0 && area_cells(g2, prev[2 * i1], prev[2 * i1 + 1], window, x0, x1, y0, y1)) {
        const uint8_t* d1 = desc1 + (size_t)i1 * 32;
        const float px = prev[2 * i1], py = prev[2 * i1 + 1];
        warp_window_keys(g2.cell_start, g2.cell_keys, g2.key_cell, ORBGPU_GRID_ROWS, x0, x1, y0, y1, [&](int idx, int c, bool valid) {
            const bool ok = valid && in_area(g2, idx, px, py, window, kp1.octave, kp1.octave);
            const unsigned m = __ballot_sync(0xffffffffu, ok);
            if (fill && ok) {
                const int pos = cand_start[i1] + total + __popc(m & ((1u << lane) - 1));
                const int dist = hamming256_ptr(d1, g2.desc + (size_t)idx * 32);
                cand_out[pos] = cand_key(dist, c, idx);
            }
            total += __popc(m);
        });
    }
    if (!fill && lane == 0) cand_count[i1] = total;
}

__global__ void k_exclusive_scan(const int* in, int n, int* out, int* total) {
    __shared__ int s_scan[32];
    int base = 0;
    for (int b0 = 0; b0 < n; b0 += blockDim.x) {
        const int i = b0 + threadIdx.x;
        const int v = i < n ? in[i] : 0;
        int tot;
        const int ex = block_exclusive_scan(v, s_scan, &tot);
        if (i < n) out[i] = base + ex;
        base += tot;
    }
    if (threadIdx.x == 0) *total = base;
}

// Pass 2: the in-order resolution of src/ORBmatcher.cc:600-677 by one warp.
// Each keypoint's choice depends on the matched distances the earlier ones
// left, so the walk is serial and its pace is memory latency: the matched
// distances and the F2 -> F1 matches live in shared memory when the launch
// gave 2 * n2 ints of it (smem_n2 >= n2), the candidate ranges are loaded 32
// keypoints at a time (keypoints without candidates are skipped in order by
// ballot), and the next keypoint's first 32 candidate keys are loaded while
// the current one is resolved.
__global__ void k_init_resolve(const orbgpu_keypoint* kps1, int n1, const orbgpu_keypoint* kps2, int n2,
                               const int* cand_start, const int* cand_count, const uint64_t* cands, float nnratio,
                               int check_ori, int smem_n2, int* matched_dist_g, int* matches21_g, int* matches12,
                               int* bin_of, int* nmatches_out) {
    extern __shared__ int s_init[];
    const int lane = threadIdx.x;
    __shared__ int hist[ORBGPU_HISTO_LENGTH];
    const bool local = smem_n2 >= n2;
    int* const matched_dist = local ? s_init : matched_dist_g;
    int* const matches21 = local ? s_init + n2 : matches21_g;
    if (lane < ORBGPU_HISTO_LENGTH) hist[lane] = 0;
    for (int i = lane; i < n2; i += 32) {
        matched_dist[i] = 0x7fffffff;
        matches21[i] = -1;
    }
    for (int i = lane; i < n1; i += 32) {
        matches12[i] = -1;
        bin_of[i] = -1;
    }
    __syncwarp();
    int nmatches = 0;
    const float factor = __fdiv_rn((float)ORBGPU_HISTO_LENGTH, 360.0f);
    for (int i0 = 0; i0 < n1; i0 += 32) {
        // the candidate ranges of keypoints i0 .. i0 + 31, one per lane
        const int mine = i0 + lane;
        const int my_s = mine < n1 ? cand_start[mine] : 0, my_c = mine < n1 ? cand_count[mine] : 0;
        unsigned live = __ballot_sync(0xffffffffu, my_c > 0);
        if (!live) continue;
        int j = __ffs(live) - 1;
        live &= live - 1;
        int s = __shfl_sync(0xffffffffu, my_s, j), cnt = __shfl_sync(0xffffffffu, my_c, j);
        uint64_t first = lane < cnt ? cands[s + lane] : ~0ull;  // the keypoint's first 32 keys
        while (true) {
            const int i1 = i0 + j;
            // the next live keypoint's range and first keys, in flight meanwhile
            const bool more = live != 0;
            int jn = 0, sn = 0, cn = 0;
            uint64_t first_n = ~0ull;
            if (more) {
                jn = __ffs(live) - 1;
                live &= live - 1;
            }
            sn = __shfl_sync(0xffffffffu, my_s, jn);
            cn = __shfl_sync(0xffffffffu, my_c, jn);
            if (more && lane < cn) first_n = cands[sn + lane];
            // best: lexicographic (dist, position); second: smallest dist of the others
            uint64_t best = ~0ull;
            int second = 0x7fffffff;
            for (int b = 0; b < cnt; b += 32) {
                uint64_t key = ~0ull;
                if (b + lane < cnt) {
                    key = b == 0 ? first : cands[s + b + lane];
                    const int dist = (int)(key >> 40);
                    const int i2 = (int)(key & 0xFFFFF);
                    if (matched_dist[i2] <= dist) key = ~0ull;
                }
                // merge (best, second) with this lane's key
                if (key < best) {
                    if (best != ~0ull) second = min(second, (int)(best >> 40));
                    best = key;
                } else if (key != ~0ull) {
                    second = min(second, (int)(key >> 40));
                }
            }
            // warp merge of (best, second)
            for (int o = 16; o > 0; o >>= 1) {
                const uint64_t ob = __shfl_xor_sync(0xffffffffu, best, o);
                const int os = __shfl_xor_sync(0xffffffffu, second, o);
                if (ob < best) {
                    second = min(os, best == ~0ull ? 0x7fffffff : (int)(best >> 40));
                    best = ob;
                } else {
                    second = min(second, min(os, ob == ~0ull ? 0x7fffffff : (int)(ob >> 40)));
                }
            }
            if (best != ~0ull) {
                const int bestDist = (int)(best >> 40);
                const int bestIdx2 = (int)(best & 0xFFFFF);
                if (bestDist <= ORBGPU_TH_LOW && (float)bestDist < __fmul_rn((float)second, nnratio)) {
                    if (lane == 0) {
                        const int prev = matches21[bestIdx2];
                        if (prev >= 0) {
                            matches12[prev] = -1;
                            nmatches--;
                        }
                        matches12[i1] = bestIdx2;
                        matches21[bestIdx2] = i1;
                        matched_dist[bestIdx2] = bestDist;
                        nmatches++;
                        if (check_ori) {
                            float rot = __fsub_rn(kps1[i1].angle, kps2[bestIdx2].angle);
                            if (rot < 0.0f) rot = __fadd_rn(rot, 360.0f);
                            int bin = (int)roundf(__fmul_rn(rot, factor));
                            if (bin == ORBGPU_HISTO_LENGTH) bin = 0;
                            bin_of[i1] = bin;
                            hist[bin]++;
                        }
                    }
                    nmatches = __shfl_sync(0xffffffffu, nmatches, 0);
                }
            }
            __syncwarp();  // lane 0's updates are seen by the next keypoint's filter
            if (!more) break;
            j = jn;
            s = sn;
            cnt = cn;
            first = first_n;
        }
    }
    if (check_ori) {
        int ind1 = -1, ind2 = -1, ind3 = -1;
        int max1 = 0, max2 = 0, max3 = 0;
        for (int i = 0; i < ORBGPU_HISTO_LENGTH; i++) {  // ComputeThreeMaxima, src/ORBmatcher.cc:2035-2077
            const int sz = hist[i];
            if (sz > max1) {
                max3 = max2; max2 = max1; max1 = sz;
                ind3 = ind2; ind2 = ind1; ind1 = i;
            } else if (sz > max2) {
                max3 = max2; max2 = sz;
                ind3 = ind2; ind2 = i;
            } else if (sz > max3) {
                max3 = sz;
                ind3 = i;
            }
        }
        if ((float)max2 < __fmul_rn(0.1f, (float)max1)) {
            ind2 = -1;
            ind3 = -1;
        } else if ((float)max3 < __fmul_rn(0.1f, (float)max1)) {
            ind3 = -1;
        }
        int removed = 0;
        for (int i1 = lane; i1 < n1; i1 += 32) {
            const int b = bin_of[i1];
            if (b < 0 || b == ind1 || b == ind2 || b == ind3) continue;
            if (matches12[i1] >= 0) {
                matches12[i1] = -1;
                removed++;
            }
        }
        nmatches -= warp_sum(removed);
    }
    if (lane == 0) *nmatches_out = nmatches;
}

// ----------------------------------------------------------------- SearchByProjection(Frame, MapPoints)
// Pass 1 (warp per map point): candidates in the scaled window over levels
// [L-1, L] that pass the stereo gate, with their distances (src/ORBmatcher.cc:84-145).
// A candidate with nnratio * dist > TH_HIGH (nnratio <= 1) can neither be
// accepted nor make an accepted best fail the ratio test, so it is left out.
__global__ void k_proj_candidates(GridDev g, const orbgpu_mappoint* mps, const uint8_t* mp_desc, int m, float th,
                                  float nnratio, const int* cand_start, int* cand_count, uint64_t* cand_out,
                                  int fill) {
    const bool drop_far = nnratio <= 1.0f;
    const int lane = threadIdx.x & 31;
    const int imp = blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5);
    if (imp >= m) return;
    const orbgpu_mappoint mp = mps[imp];
    int total = 0;
    if (mp.track_in_view && !mp.bad && mp.track_scale_level >= 0 && mp.track_scale_level < 16) {
        const int level = mp.track_scale_level;
        float r = mp.view_cos > 0.998f ? 2.5f : 4.0f;  // RadiusByViewingCos, src/ORBmatcher.cc:186-193
        if (th != 1.0f) r = __fmul_rn(r, th);
        const float radius = __fmul_rn(r, g.scale[level]);
        int x0, x1, y0, y1;
        if (area_cells(g, mp.proj_x, mp.proj_y, radius, x0, x1, y0, y1)) {
            const uint8_t* dmp = mp_desc + (size_t)imp * 32;
            warp_window_keys(g.cell_start, g.cell_keys, g.key_cell, ORBGPU_GRID_ROWS, x0, x1, y0, y1, [&](int idx, int c, bool valid) {
                bool ok = valid && in_area(g, idx, mp.proj_x, mp.proj_y, radius, level - 1, level);
                if (ok && g.uright && g.uright[idx] > 0) {
                    const float er = fabsf(__fsub_rn(mp.proj_xr, g.uright[idx]));
                    if (er > radius) ok = false;
                }
                int dist = 256;
                if (ok) {
                    dist = hamming256_ptr(dmp, g.desc + (size_t)idx * 32);
                    ok = !(drop_far && __fmul_rn(nnratio, (float)dist) > (float)ORBGPU_TH_HIGH);
                }
                const unsigned msk = __ballot_sync(0xffffffffu, ok);
                if (fill && ok) {
                    const int pos = cand_start[imp] + total + __popc(msk & ((1u << lane) - 1));
                    cand_out[pos] = cand_key(dist, c, idx);
                }
                total += __popc(msk);
            });
        }
    }
    if (!fill && lane == 0) cand_count[imp] = total;
}

// Pass 2: in-order resolution (src/ORBmatcher.cc:117-180) by one warp.
// claimed[] starts with the caller's pre-claimed keypoints.
__global__ void k_proj_resolve(GridDev g, int m, const int* cand_start, const int* cand_count, const uint64_t* cands,
                               float nnratio, int* match_out, int* nmatches_out, const int* converged_flags) {
    if (converged_flags && converged_flags[PROJ_ROUNDS - 1] == 0) return;
    const int lane = threadIdx.x;
    int nmatches = 0;
    for (int imp = 0; imp < m; imp++) {
        const int s = cand_start[imp], cnt = cand_count[imp];
        if (cnt == 0) continue;
        uint64_t best = ~0ull, second = ~0ull;
        for (int b = 0; b < cnt; b += 32) {
            uint64_t key = ~0ull;
            if (b + lane < cnt) {
                key = cands[s + b + lane];
                const int idx = (int)(key & 0xFFFFF);
                if (match_out[idx] != -1 || (int)(key >> 40) >= 256) key = ~0ull;
            }
            if (key < best) {
                second = best;
                best = key;
            } else if (key < second) {
                second = key;
            }
        }
        for (int o = 16; o > 0; o >>= 1) {
            const uint64_t ob = __shfl_xor_sync(0xffffffffu, best, o);
            const uint64_t os = __shfl_xor_sync(0xffffffffu, second, o);
            if (ob < best) {
                second = min(best, os);
                best = ob;
            } else {
                second = min(second, ob);
            }
        }
        if (best == ~0ull) continue;
        const int bestDist = (int)(best >> 40);
        const int bestIdx = (int)(best & 0xFFFFF);
        const int bestLevel = g.kps[bestIdx].octave;
        const int bestDist2 = second == ~0ull ? 256 : (int)(second >> 40);
        const int bestLevel2 = second == ~0ull ? -1 : g.kps[(int)(second & 0xFFFFF)].octave;
        if (bestDist <= ORBGPU_TH_HIGH) {
            if (bestLevel == bestLevel2 && (float)bestDist > __fmul_rn(nnratio, (float)bestDist2)) continue;
            if (lane == 0) match_out[bestIdx] = imp;
            nmatches++;
        }
        __syncwarp();
    }
    if (lane == 0) *nmatches_out = nmatches;
}

// Parallel resolution of the same search by fixed-point rounds (the scheme
// of the batched search): round r evaluates every map point against the
// claims of round r-1's results; when a round changes nothing the results
// equal the sequential ones.  Pre-claimed keypoints (match_out == -2) are
// always excluded.  k_proj_resolve replays serially if no round converged.
__global__ void k_proj_round(GridDev g, int m, const int* cand_start, const int* cand_count, const uint64_t* cands,
                             float nnratio, int round, int* claims3, int* res, int* changed, const int* pre) {
    const int lane = threadIdx.x & 31;
    const int local = blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5);
    const int nwarps = gridDim.x * (blockDim.x >> 5);
    if (round > 0 && changed[round - 1] == 0) return;
    const int n = g.n;
    int* claims_r = claims3 + (size_t)((round + 0) % 3) * n;
    int* claims_w = claims3 + (size_t)((round + 1) % 3) * n;
    int* claims_z = claims3 + (size_t)((round + 2) % 3) * n;
    for (int i = local * 32 + lane; i < n; i += nwarps * 32) claims_z[i] = PROJ_NONE;
    if (local >= m) return;
    const int s = cand_start[local], cnt = cand_count[local];
    uint64_t best = ~0ull, second = ~0ull;
    for (int b = 0; b < cnt; b += 32) {
        uint64_t key = ~0ull;
        if (b + lane < cnt) {
            key = cands[s + b + lane];
            const int idx = (int)(key & 0xFFFFF);
            if (pre[idx] == -2 || claims_r[idx] < local || (int)(key >> 40) >= 256) key = ~0ull;
        }
        if (key < best) {
            second = best;
            best = key;
        } else if (key < second) {
            second = key;
        }
    }
    for (int o = 16; o > 0; o >>= 1) {
        const uint64_t ob = __shfl_xor_sync(0xffffffffu, best, o);
        const uint64_t os = __shfl_xor_sync(0xffffffffu, second, o);
        if (ob < best) {
            second = best < os ? best : os;
            best = ob;
        } else {
            second = second < ob ? second : ob;
        }
    }
    int r = -1;
    if (best != ~0ull) {
        const int bestDist = (int)(best >> 40);
        const int bestIdx = (int)(best & 0xFFFFF);
        const int bestLevel = g.kps[bestIdx].octave;
        const int bestDist2 = second == ~0ull ? 256 : (int)(second >> 40);
        const int bestLevel2 = second == ~0ull ? -1 : g.kps[(int)(second & 0xFFFFF)].octave;
        if (bestDist <= ORBGPU_TH_HIGH &&
            !(bestLevel == bestLevel2 && (float)bestDist > __fmul_rn(nnratio, (float)bestDist2)))
            r = bestIdx;
    }
    if (lane == 0) {
        if (res[local] != r) changed[round] = 1;
        res[local] = r;
        if (r >= 0) atomicMin(&claims_w[r], local);
    }
}

// Converged rounds: write the matches; otherwise leave match_out for the
// serial replay.
__global__ void k_proj_finish(int m, const int* changed, const int* res, int* match_out, int* nmatches_out) {
    if (changed[PROJ_ROUNDS - 1] != 0) return;
    int nm = 0;
    for (int i = threadIdx.x; i < m; i += blockDim.x) {
        const int r = res[i];
        if (r >= 0) {
            match_out[r] = i;
            nm++;
        }
    }
    atomicAdd(nmatches_out, nm);
}

__global__ void k_init_match_out(const uint8_t* claimed, int n, int* match_out) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) match_out[i] = (claimed && claimed[i]) ? -2 : -1;
}

// ----------------------------------------------------------------- SearchByProjection(Frame, LastFrame)
// src/ORBmatcher.cc:1710-1879.  Per LastFrame map point (one warp): the pose
// algebra with the reference's rounding (3 x 3 float product accumulated in
// double and stored as float, then a float addition; 1.0 / z in double), the
// window over the current grid with the motion-dependent level range, the
// stereo gate, and the candidates whose distance can be accepted
// (<= TH_HIGH: with no ratio test the first minimum is the answer, and a
// minimum above TH_HIGH is rejected either way).
struct FrameMotionDev {
    float T[12];
    float fx, fy, cx, cy, bf;
    float maxX, maxY;
    int level_mode;  // 1 forward, 2 backward, 0 neither
};

__device__ __forceinline__ float pose_row(const float* row, float X0, float X1, float X2) {
    double s = __dadd_rn(0.0, __dmul_rn((double)row[0], (double)X0));
    s = __dadd_rn(s, __dmul_rn((double)row[1], (double)X1));
    s = __dadd_rn(s, __dmul_rn((double)row[2], (double)X2));
    return __fadd_rn(__double2float_rn(s), row[3]);
}

__global__ void k_pf_candidates(GridDev g, FrameMotionDev mo, const orbgpu_keypoint* last_kps,
                                const orbgpu_frame_mappoint* mps, const uint8_t* mp_desc, int m, float th,
                                const int* cand_start, int* cand_count, uint64_t* cand_out, int fill) {
    const int lane = threadIdx.x & 31;
    const int i = blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5);
    if (i >= m) return;
    const orbgpu_frame_mappoint mp = mps[i];
    int total = 0;
    const int oct = last_kps[i].octave;
    bool live = (mp.flags & ORBGPU_MP_PRESENT) && !(mp.flags & ORBGPU_MP_OUTLIER) && oct >= 0 && oct < 16;
    float u = 0.f, v = 0.f, invzc = 0.f;
    if (live) {
        const float xc = pose_row(mo.T, mp.x, mp.y, mp.z);
        const float yc = pose_row(mo.T + 4, mp.x, mp.y, mp.z);
        const float zc = pose_row(mo.T + 8, mp.x, mp.y, mp.z);
        invzc = __double2float_rn(__ddiv_rn(1.0, (double)zc));
        u = __fadd_rn(__fmul_rn(__fmul_rn(mo.fx, xc), invzc), mo.cx);
        v = __fadd_rn(__fmul_rn(__fmul_rn(mo.fy, yc), invzc), mo.cy);
        // a non-finite projection finds no grid cell in the reference
        live = !(invzc < 0.f) && isfinite(u) && isfinite(v) && !(u < g.minX || u > mo.maxX) &&
               !(v < g.minY || v > mo.maxY);
    }
    if (live) {
        const float radius = __fmul_rn(th, g.scale[oct]);
        int minL, maxL;
        if (mo.level_mode == 1) {
            minL = oct;
            maxL = -1;
        } else if (mo.level_mode == 2) {
            minL = 0;
            maxL = oct;
        } else {
            minL = oct - 1;
            maxL = oct + 1;
        }
        int x0, x1, y0, y1;
        if (area_cells(g, u, v, radius, x0, x1, y0, y1)) {
            const uint8_t* dmp = mp_desc + (size_t)i * 32;
            const float ur = __fsub_rn(u, __fmul_rn(mo.bf, invzc));
            warp_window_keys(g.cell_start, g.cell_keys, g.key_cell, ORBGPU_GRID_ROWS, x0, x1, y0, y1, [&](int idx, int c, bool valid) {
                bool ok = valid && in_area(g, idx, u, v, radius, minL, maxL);
                if (ok && g.uright && g.uright[idx] > 0) {
                    const float er = fabsf(__fsub_rn(ur, g.uright[idx]));
                    if (er > radius) ok = false;
                }
                int dist = 256;
                if (ok) {
                    dist = hamming256_ptr(dmp, g.desc + (size_t)idx * 32);
                    ok = dist <= ORBGPU_TH_HIGH;
                }
                const unsigned msk = __ballot_sync(0xffffffffu, ok);
                if (fill && ok) {
                    const int pos = cand_start[i] + total + __popc(msk & ((1u << lane) - 1));
                    cand_out[pos] = cand_key(dist, c, idx);
                }
                total += __popc(msk);
            });
        }
    }
    if (!fill && lane == 0) cand_count[i] = total;
}

// ----------------------------------------------------------------- SearchByProjection(Frame, KeyFrame)
// src/ORBmatcher.cc:1891-2010 (relocalisation): the keyframe's map points
// that are usable (not NULL, not bad, not in sAlreadyFound) in keyframe order.
// Per map point (one warp): Rcw * X + tcw as in the frame-to-frame search
// (no depth test here), the projection, the distance invariance, the level
// MapPoint::PredictScale gives (thresholds of orbgpu_frustum_frame_init), the
// window of levels level - 1 .. level + 1 with radius th * scale[level], and
// the candidates at distance <= ORBdist (no ratio test: the first minimum is
// the answer, and a minimum above ORBdist is rejected either way).
struct KeyframeProjDev {
    float T[12];
    float Ow[3];
    float fx, fy, cx, cy;
    float maxX, maxY;
    int nlevels;
    float level_above[15];
    int orbdist;
    // 1: SearchByProjection(KeyFrame*, Scw, vpPoints, vpMatched, th)
    // (src/ORBmatcher.cc:423-560): depth test, IsInImage bounds, viewing angle,
    // levels level - 1 .. level, u = fx * (x * invz) + cx
    int sim3;
    // with sim3: Fuse(KeyFrame*, vpMapPoints, th) (src/ORBmatcher.cc:1107-1245)
    // adds the reprojection-error gate of every candidate (stereo with ur)
    int fuse;
    float bf;
    float inv_sigma2[16];
    // Fuse(KeyFrame*, Scw, ...) (src/ORBmatcher.cc:1290-1380): invz = 1.0 / z
    // in double, rounded to float
    int invz_double;
    // SearchBySim3 (src/ORBmatcher.cc:1441-1640): a second transform T2
    // applied to the camera coordinates (the Sim3 between the keyframes), the
    // depth for the distance invariance is |p3Dc| and there is no viewing
    // angle test
    int chain;
    float T2[12];
};

__global__ void k_pkf_candidates(GridDev g, KeyframeProjDev kp, const orbgpu_mappoint_geometry* mps,
                                 const uint8_t* usable, const uint8_t* mp_desc, int m, float th,
                                 const int* cand_start, int* cand_count, uint64_t* cand_out, int fill) {
    const int lane = threadIdx.x & 31;
    const int i = blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5);
    if (i >= m) return;
    int total = 0;
    bool live = usable[i] == 1;
    float u = 0.f, v = 0.f, ur_f = 0.f;
    int level = 0;
    if (live) {
        const orbgpu_mappoint_geometry mp = mps[i];
        float xc = pose_row(kp.T, mp.x, mp.y, mp.z);
        float yc = pose_row(kp.T + 4, mp.x, mp.y, mp.z);
        float zc = pose_row(kp.T + 8, mp.x, mp.y, mp.z);
        if (kp.chain) {
            const float x1 = xc, y1 = yc, z1 = zc;
            xc = pose_row(kp.T2, x1, y1, z1);
            yc = pose_row(kp.T2 + 4, x1, y1, z1);
            zc = pose_row(kp.T2 + 8, x1, y1, z1);
        }
        if (kp.sim3) {
            const float invz = kp.invz_double ? __double2float_rn(__ddiv_rn(1.0, (double)zc)) : __fdiv_rn(1.0f, zc);
            u = __fadd_rn(__fmul_rn(kp.fx, __fmul_rn(xc, invz)), kp.cx);
            v = __fadd_rn(__fmul_rn(kp.fy, __fmul_rn(yc, invz)), kp.cy);
            ur_f = __fsub_rn(u, __fmul_rn(kp.bf, invz));
            // KeyFrame::IsInImage (upper bounds exclusive); NaN fails it
            live = !(zc < 0.0f) && u >= g.minX && u < kp.maxX && v >= g.minY && v < kp.maxY;
        } else {
            const float invzc = __double2float_rn(__ddiv_rn(1.0, (double)zc));
            u = __fadd_rn(__fmul_rn(__fmul_rn(kp.fx, xc), invzc), kp.cx);
            v = __fadd_rn(__fmul_rn(__fmul_rn(kp.fy, yc), invzc), kp.cy);
            // a non-finite projection finds no grid cell in the reference
            live = isfinite(u) && isfinite(v) && !(u < g.minX || u > kp.maxX) && !(v < g.minY || v > kp.maxY);
        }
        if (live) {
            // PO = X - Ow, or the camera coordinates themselves for SearchBySim3
            const float po0 = kp.chain ? xc : __fsub_rn(mp.x, kp.Ow[0]);
            const float po1 = kp.chain ? yc : __fsub_rn(mp.y, kp.Ow[1]);
            const float po2 = kp.chain ? zc : __fsub_rn(mp.z, kp.Ow[2]);
            double ss = __dmul_rn((double)po0, (double)po0);
            ss = __dadd_rn(ss, __dmul_rn((double)po1, (double)po1));
            ss = __dadd_rn(ss, __dmul_rn((double)po2, (double)po2));
            const float dist = (float)__dsqrt_rn(ss);
            live = !(dist < __fmul_rn(0.8f, mp.min_distance) || dist > __fmul_rn(1.2f, mp.max_distance));
            if (live && kp.sim3 && !kp.chain) {
                // PO.dot(Pn) < 0.5 * dist, in double
                double dp = __dmul_rn((double)po0, (double)mp.nx);
                dp = __dadd_rn(dp, __dmul_rn((double)po1, (double)mp.ny));
                dp = __dadd_rn(dp, __dmul_rn((double)po2, (double)mp.nz));
                live = !(dp < __dmul_rn(0.5, (double)dist));
            }
            const float ratio = __fdiv_rn(mp.max_distance, dist);
            for (int n = 0; n < kp.nlevels - 1; n++) level += ratio > kp.level_above[n] ? 1 : 0;
        }
    }
    if (live) {
        const float radius = __fmul_rn(th, g.scale[level]);
        int x0, x1, y0, y1;
        if (area_cells(g, u, v, radius, x0, x1, y0, y1)) {
            const uint8_t* dmp = mp_desc + (size_t)i * 32;
            warp_window_keys(g.cell_start, g.cell_keys, g.key_cell, ORBGPU_GRID_ROWS, x0, x1, y0, y1,
                             [&](int idx, int c, bool valid) {
                bool ok;
                if (kp.sim3) {
                    // KeyFrame::GetFeaturesInArea (src/KeyFrame.cc:785-830): a square
                    // window (|dx| < r and |dy| < r; Frame's is a disc), then the
                    // levels predicted - 1 .. predicted
                    const orbgpu_keypoint& kq = g.kps[idx];
                    ok = valid && kq.octave >= level - 1 && kq.octave <= level &&
                         fabsf(__fsub_rn(kq.x, u)) < radius && fabsf(__fsub_rn(kq.y, v)) < radius;
                } else {
                    ok = valid && in_area(g, idx, u, v, radius, level - 1, level + 1);
                }
                if (ok && kp.fuse) {
                    // chi-square gates of Fuse: 7.8 with the right coordinate, 5.99 without
                    const orbgpu_keypoint& k = g.kps[idx];
                    const float ex = __fsub_rn(u, k.x), ey = __fsub_rn(v, k.y);
                    float e2 = __fadd_rn(__fmul_rn(ex, ex), __fmul_rn(ey, ey));
                    const bool stereo = g.uright && g.uright[idx] >= 0.0f;
                    if (stereo) {
                        const float er = __fsub_rn(ur_f, g.uright[idx]);
                        e2 = __fadd_rn(e2, __fmul_rn(er, er));
                    }
                    ok = !((double)__fmul_rn(e2, kp.inv_sigma2[k.octave & 15]) > (stereo ? 7.8 : 5.99));
                }
                int dist = 256;
                if (ok) {
                    dist = hamming256_ptr(dmp, g.desc + (size_t)idx * 32);
                    ok = dist <= kp.orbdist;
                }
                const unsigned msk = __ballot_sync(0xffffffffu, ok);
                if (fill && ok) {
                    const int pos = cand_start[i] + total + __popc(msk & ((1u << lane) - 1));
                    cand_out[pos] = cand_key(dist, c, idx);
                }
                total += __popc(msk);
            });
        }
    }
    if (!fill && lane == 0) cand_count[i] = total;
}

// Fixed-point round r of the in-order assignment: map point i takes its
// first minimum among candidates not held by an observed map point j < i of
// round r-1's results (an owner without observations blocks nothing,
// src/ORBmatcher.cc:1800-1802; with mps NULL every owner blocks, as in
// SearchByProjection(Frame&, KeyFrame*, ...)).  A round that changes nothing
// equals the sequential result.
__global__ void k_pf_round(int n, int m, const int* cand_start, const int* cand_count, const uint64_t* cands,
                           const orbgpu_frame_mappoint* mps, int round, int* claims3, int* res, int* changed,
                           const int* pre) {
    const int lane = threadIdx.x & 31;
    const int local = blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5);
    const int nwarps = gridDim.x * (blockDim.x >> 5);
    if (round > 0 && changed[round - 1] == 0) return;
    int* claims_r = claims3 + (size_t)((round + 0) % 3) * n;
    int* claims_w = claims3 + (size_t)((round + 1) % 3) * n;
    int* claims_z = claims3 + (size_t)((round + 2) % 3) * n;
    for (int k = local * 32 + lane; k < n; k += nwarps * 32) claims_z[k] = PROJ_NONE;
    if (local >= m) return;
    const int s = cand_start[local], cnt = cand_count[local];
    uint64_t best = ~0ull;
    for (int b = lane; b < cnt; b += 32) {
        const uint64_t key = cands[s + b];
        const int idx = (int)(key & 0xFFFFF);
        if (pre[idx] != -2 && !(claims_r[idx] < local) && key < best) best = key;
    }
    for (int o = 16; o > 0; o >>= 1) {
        const uint64_t ob = __shfl_xor_sync(0xffffffffu, best, o);
        best = ob < best ? ob : best;
    }
    const int r = best == ~0ull ? -1 : (int)(best & 0xFFFFF);
    if (lane == 0) {
        if (res[local] != r) changed[round] = 1;
        res[local] = r;
        if (r >= 0 && (!mps || (mps[local].flags & ORBGPU_MP_OBSERVED))) atomicMin(&claims_w[r], local);
    }
}

// Sequential assignment when no round converged (one warp).
__global__ void k_pf_serial(int n, int m, const int* cand_start, const int* cand_count, const uint64_t* cands,
                            const orbgpu_frame_mappoint* mps, const int* changed, int* res, int* blocked,
                            const int* pre) {
    if (changed[PROJ_ROUNDS - 1] == 0) return;
    const int lane = threadIdx.x;
    for (int k = lane; k < n; k += 32) blocked[k] = pre[k] == -2;
    __syncwarp();
    for (int i = 0; i < m; i++) {
        const int s = cand_start[i], cnt = cand_count[i];
        uint64_t best = ~0ull;
        for (int b = lane; b < cnt; b += 32) {
            const uint64_t key = cands[s + b];
            if (!blocked[(int)(key & 0xFFFFF)] && key < best) best = key;
        }
        for (int o = 16; o > 0; o >>= 1) {
            const uint64_t ob = __shfl_xor_sync(0xffffffffu, best, o);
            best = ob < best ? ob : best;
        }
        const int r = best == ~0ull ? -1 : (int)(best & 0xFFFFF);
        if (lane == 0) {
            res[i] = r;
            if (r >= 0 && (!mps || (mps[i].flags & ORBGPU_MP_OBSERVED))) blocked[r] = 1;
        }
        __syncwarp();
    }
}

// Owners (the last map point that assigned each keypoint), the rotation
// histogram of every assignment (src/ORBmatcher.cc:1847-1857), the three
// maxima and the resets (:1862-1876), and the output codes.  One block.
__global__ void __launch_bounds__(1024) k_pf_finish(int n, int m, const int* res, const orbgpu_keypoint* last_kps,
                                                    const orbgpu_keypoint* cur_kps, int check_ori, int* owner,
                                                    int* bin_of, int* nulled, int* match_out, int* nmatches_out) {
    __shared__ int hist[ORBGPU_HISTO_LENGTH];
    __shared__ int s_nm, s_ind[3];
    if (threadIdx.x < ORBGPU_HISTO_LENGTH) hist[threadIdx.x] = 0;
    if (threadIdx.x == 0) s_nm = 0;
    for (int k = threadIdx.x; k < n; k += blockDim.x) {
        owner[k] = -1;
        nulled[k] = 0;
    }
    __syncthreads();
    const float factor = __fdiv_rn((float)ORBGPU_HISTO_LENGTH, 360.0f);
    int nm = 0;
    for (int i = threadIdx.x; i < m; i += blockDim.x) {
        const int r = res[i];
        int bin = -1;
        if (r >= 0) {
            nm++;
            atomicMax(&owner[r], i);
            if (check_ori) {
                float rot = __fsub_rn(last_kps[i].angle, cur_kps[r].angle);
                if (rot < 0.0f) rot = __fadd_rn(rot, 360.0f);
                bin = (int)roundf(__fmul_rn(rot, factor));
                if (bin == ORBGPU_HISTO_LENGTH) bin = 0;
                atomicAdd(&hist[bin], 1);
            }
        }
        bin_of[i] = bin;
    }
    atomicAdd(&s_nm, nm);
    __syncthreads();
    if (threadIdx.x == 0) {
        int ind1 = -1, ind2 = -1, ind3 = -1;
        if (check_ori) {
            int max1 = 0, max2 = 0, max3 = 0;
            for (int b = 0; b < ORBGPU_HISTO_LENGTH; b++) {  // ComputeThreeMaxima, src/ORBmatcher.cc:2035-2077
                const int sz = hist[b];
                if (sz > max1) {
                    max3 = max2; max2 = max1; max1 = sz;
                    ind3 = ind2; ind2 = ind1; ind1 = b;
                } else if (sz > max2) {
                    max3 = max2; max2 = sz;
                    ind3 = ind2; ind2 = b;
                } else if (sz > max3) {
                    max3 = sz;
                    ind3 = b;
                }
            }
            if ((float)max2 < __fmul_rn(0.1f, (float)max1)) {
                ind2 = -1;
                ind3 = -1;
            } else if ((float)max3 < __fmul_rn(0.1f, (float)max1)) {
                ind3 = -1;
            }
        }
        s_ind[0] = ind1;
        s_ind[1] = ind2;
        s_ind[2] = ind3;
    }
    __syncthreads();
    if (check_ori) {
        int removed = 0;
        for (int i = threadIdx.x; i < m; i += blockDim.x) {
            const int b = bin_of[i];
            if (b < 0 || b == s_ind[0] || b == s_ind[1] || b == s_ind[2]) continue;
            nulled[res[i]] = 1;
            removed++;
        }
        atomicSub(&s_nm, removed);
    }
    __syncthreads();
    for (int k = threadIdx.x; k < n; k += blockDim.x) {
        const int pre = match_out[k];
        match_out[k] = nulled[k] ? -4 : owner[k] >= 0 ? owner[k] : pre;
    }
    if (threadIdx.x == 0) *nmatches_out = s_nm;
}

// ----------------------------------------------------------------- stereo
// (the device functions are in orbgpu_stereo.cuh)
__global__ void k_stereo_rows_count(const orbgpu_keypoint* kpsR, int nR, StereoLevels lv, int nRows, int* row_count) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    int lo, hi;
    if (i >= nR || !stereo_rows_of(kpsR[i], lv, nRows, lo, hi)) return;
    for (int yi = lo; yi <= hi; yi++) atomicAdd(&row_count[yi], 1);
}

__global__ void k_stereo_rows_fill(const orbgpu_keypoint* kpsR, int nR, StereoLevels lv, int nRows, int* cursor,
                                   int* row_keys) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    int lo, hi;
    if (i >= nR || !stereo_rows_of(kpsR[i], lv, nRows, lo, hi)) return;
    for (int yi = lo; yi <= hi; yi++) row_keys[atomicAdd(&cursor[yi], 1)] = i;
}

// Frame::ComputeStereoMatches per left keypoint (src/Frame.cc:884-1064), one warp each.
__global__ void k_stereo_match(const orbgpu_keypoint* kpsL, const uint8_t* descL, int nL, const orbgpu_keypoint* kpsR,
                               const uint8_t* descR, StereoLevels lv, int nRows, const int* row_start,
                               const int* row_keys, float bf, float fx, float* uright, float* depth, int* sad_out,
                               int* status) {
    const int iL = blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5);
    if (iL >= nL) return;
    stereo_match_warp(iL, kpsL, descL, kpsR, descR, lv, nRows, row_start, row_keys, bf, fx, uright, depth, sad_out,
                      status);
}

// Median cut (src/Frame.cc:1069-1081): one block.
__global__ void k_stereo_median(int nL, const int* sad, float* uright, float* depth, int* sort_buf, int cap,
                                int* n_valid) {
    stereo_median_block(nL, sad, uright, depth, sort_buf, cap, n_valid);
}

// ----------------------------------------------------------------- distance batch
__global__ void k_descriptor_distance(const uint8_t* a, const uint8_t* b, int n, int* out) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) out[i] = hamming256_ptr(a + (size_t)i * 32, b + (size_t)i * 32);
}

}  // namespace orbgpu

using namespace orbgpu;

// ----------------------------------------------------------------- host side
struct orbgpu_matcher {
    float nnratio;
    int check_ori;
    cudaStream_t stream = nullptr;
    bool own_stream = false;
    // scratch (grown on demand)
    void* scratch = nullptr;
    size_t scratch_bytes = 0;
    int* h_pinned = nullptr;
};

namespace {

struct Staged {
    const orbgpu_keypoint* kps = nullptr;
    const uint8_t* desc = nullptr;
    const float* uright = nullptr;
};

struct Bump {
    uint8_t* base;
    size_t off = 0, cap;
    template <typename T> T* take(size_t n) {
        off = (off + 255) & ~(size_t)255;
        T* p = (T*)(base + off);
        off += n * sizeof(T);
        return p;
    }
};

int ensure_scratch(orbgpu_matcher* m, size_t bytes) {
    if (bytes <= m->scratch_bytes) return ORBGPU_OK;
    ORBGPU_CUDA_TRY(cudaStreamSynchronize(m->stream));
    if (m->scratch) cudaFree(m->scratch);
    m->scratch = nullptr;
    m->scratch_bytes = 0;
    ORBGPU_CUDA_TRY(cudaMalloc(&m->scratch, bytes));
    m->scratch_bytes = bytes;
    return ORBGPU_OK;
}

// Device copies of a frame's arrays (or the caller's device pointers).
int stage_frame(orbgpu_matcher* m, const orbgpu_frame* f, Bump& b, Staged& s) {
    if (f->mem == ORBGPU_MEM_DEVICE) {
        s.kps = f->keypoints;
        s.desc = f->descriptors;
        s.uright = f->uright;
        return ORBGPU_OK;
    }
    orbgpu_keypoint* k = b.take<orbgpu_keypoint>(std::max(1, f->n));
    uint8_t* d = b.take<uint8_t>((size_t)std::max(1, f->n) * 32);
    if (f->n > 0) {
        ORBGPU_CUDA_TRY(cudaMemcpyAsync(k, f->keypoints, sizeof(orbgpu_keypoint) * f->n, cudaMemcpyHostToDevice, m->stream));
        ORBGPU_CUDA_TRY(cudaMemcpyAsync(d, f->descriptors, 32 * (size_t)f->n, cudaMemcpyHostToDevice, m->stream));
    }
    s.kps = k;
    s.desc = d;
    s.uright = nullptr;
    if (f->uright) {
        float* u = b.take<float>(std::max(1, f->n));
        if (f->n > 0) ORBGPU_CUDA_TRY(cudaMemcpyAsync(u, f->uright, sizeof(float) * f->n, cudaMemcpyHostToDevice, m->stream));
        s.uright = u;
    }
    return ORBGPU_OK;
}

size_t frame_stage_bytes(const orbgpu_frame* f) {
    if (f->mem == ORBGPU_MEM_DEVICE) return 0;
    return (size_t)std::max(1, f->n) * (sizeof(orbgpu_keypoint) + 32 + 4) + 1024;
}

size_t grid_bytes(int n) { return (size_t)(3 * 3072 + 8 + 2 * std::max(1, n)) * sizeof(int) + 2048; }

// AssignFeaturesToGrid (src/Frame.cc:399-423) on the device.
int build_grid(orbgpu_matcher* m, const orbgpu_frame* f, const Staged& s, Bump& b, GridDev& g) {
    const int ncell = ORBGPU_GRID_COLS * ORBGPU_GRID_ROWS;
    int* cell_count = b.take<int>(ncell);
    int* cell_start = b.take<int>(ncell + 1);
    int* cursor = b.take<int>(ncell);
    int* key_cell = b.take<int>(std::max(1, f->n));
    int* cell_keys = b.take<int>(std::max(1, f->n));
    g.kps = s.kps;
    g.desc = s.desc;
    g.uright = s.uright;
    g.n = f->n;
    g.minX = 0.0f;
    g.minY = 0.0f;
    g.invW = static_cast<float>(ORBGPU_GRID_COLS) / static_cast<float>((float)f->width - 0.0f);
    g.invH = static_cast<float>(ORBGPU_GRID_ROWS) / static_cast<float>((float)f->height - 0.0f);
    g.cell_start = cell_start;
    g.cell_keys = cell_keys;
    g.key_cell = key_cell;
    for (int l = 0; l < 16; l++) g.scale[l] = l < f->nlevels ? f->scale_factors[l] : 1.0f;
    ORBGPU_CUDA_TRY(cudaMemsetAsync(cell_count, 0, sizeof(int) * ncell, m->stream));
    if (f->n > 0) k_grid_count<<<(f->n + 255) / 256, 256, 0, m->stream>>>(s.kps, f->n, g.minX, g.minY, g.invW, g.invH, key_cell, cell_count);
    k_grid_scan<<<1, 1024, 0, m->stream>>>(cell_count, cell_start, cursor);
    if (f->n > 0) k_grid_fill<<<(f->n + 255) / 256, 256, 0, m->stream>>>(key_cell, f->n, cursor, cell_keys);
    ORBGPU_CUDA_TRY(cudaGetLastError());
    return ORBGPU_OK;
}

bool frame_ok(const orbgpu_frame* f) {
    return f && f->n >= 0 && f->n < (1 << 20) && f->width > 0 && f->height > 0 && f->nlevels >= 1 &&
           f->nlevels <= 16 && (f->n == 0 || (f->keypoints && f->descriptors));
}

}  // namespace

extern "C" int orbgpu_matcher_create(float nnratio, int check_orientation, void* stream, orbgpu_matcher** out) {
    if (!out) return ORBGPU_ERR_BAD_ARG;
    int dev;
    ORBGPU_CUDA_TRY(cudaGetDevice(&dev));
    orbgpu_matcher* m = new orbgpu_matcher();
    m->nnratio = nnratio;
    m->check_ori = check_orientation;
    if (stream) m->stream = (cudaStream_t)stream;
    else {
        if (cudaStreamCreateWithFlags(&m->stream, cudaStreamNonBlocking) != cudaSuccess) {
            delete m;
            return ORBGPU_ERR_CUDA;
        }
        m->own_stream = true;
    }
    if (cudaMallocHost(&m->h_pinned, 64) != cudaSuccess) {
        orbgpu_matcher_destroy(m);
        return ORBGPU_ERR_OOM;
    }
    *out = m;
    return ORBGPU_OK;
}

extern "C" int orbgpu_matcher_destroy(orbgpu_matcher* m) {
    if (!m) return ORBGPU_OK;
    if (m->stream) cudaStreamSynchronize(m->stream);
    cudaFree(m->scratch);
    cudaFreeHost(m->h_pinned);
    if (m->own_stream) cudaStreamDestroy(m->stream);
    delete m;
    return ORBGPU_OK;
}

// Runs the two-pass candidate listing: count, scan, fill.  Returns the
// device candidate arrays in (start, count, keys).
template <typename Launch>
static int candidate_lists(orbgpu_matcher* m, int nq, Bump& b, Launch launch, int*& start, int*& count,
                           uint64_t*& keys, int& total) {
    count = b.take<int>(std::max(1, nq));
    start = b.take<int>(std::max(1, nq));
    int* d_total = b.take<int>(1);
    launch((const int*)nullptr, count, (uint64_t*)nullptr, 0);
    k_exclusive_scan<<<1, 1024, 0, m->stream>>>(count, nq, start, d_total);
    ORBGPU_CUDA_TRY(cudaMemcpyAsync(m->h_pinned, d_total, sizeof(int), cudaMemcpyDeviceToHost, m->stream));
    ORBGPU_CUDA_TRY(cudaStreamSynchronize(m->stream));
    total = m->h_pinned[0];
    const size_t need = b.off + 256 + sizeof(uint64_t) * (size_t)std::max(1, total);
    if (need > b.cap) return ORBGPU_ERR_CAPACITY;
    keys = b.take<uint64_t>(std::max(1, total));
    launch((const int*)start, count, keys, 1);
    ORBGPU_CUDA_TRY(cudaGetLastError());
    return ORBGPU_OK;
}

extern "C" int orbgpu_search_for_initialization(orbgpu_matcher* m, const orbgpu_frame* f1, const orbgpu_frame* f2,
                                                float* prev_matched, int* matches12, int window_size, int* nmatches) {
    if (!m || !frame_ok(f1) || !frame_ok(f2) || !prev_matched || !matches12 || !nmatches) return ORBGPU_ERR_BAD_ARG;
    const int n1 = f1->n, n2 = f2->n;
    *nmatches = 0;
    for (int i = 0; i < n1; i++) matches12[i] = -1;
    if (n1 == 0) return ORBGPU_OK;
    // generous scratch: every F1 key may see every F2 key
    size_t est = frame_stage_bytes(f1) + frame_stage_bytes(f2) + grid_bytes(n2) +
                 (size_t)n1 * 2 * 3 * sizeof(int) + (size_t)n2 * 2 * sizeof(int) + 64 * 1024 +
                 sizeof(uint64_t) * (size_t)n1 * std::max(1, std::min(n2, 4096));
    for (int attempt = 0; attempt < 2; attempt++) {
        int rc = ensure_scratch(m, est);
        if (rc) return rc;
        Bump b{(uint8_t*)m->scratch, 0, m->scratch_bytes};
        Staged s1, s2;
        if ((rc = stage_frame(m, f1, b, s1)) || (rc = stage_frame(m, f2, b, s2))) return rc;
        GridDev g2;
        if ((rc = build_grid(m, f2, s2, b, g2))) return rc;
        float* d_prev = b.take<float>(2 * n1);
        ORBGPU_CUDA_TRY(cudaMemcpyAsync(d_prev, prev_matched, sizeof(float) * 2 * n1, cudaMemcpyHostToDevice, m->stream));
        int *start, *count, total;
        uint64_t* keys;
        const float window = (float)window_size;
        auto launch = [&](const int* st, int* cnt, uint64_t* out, int fill) {
            const int wpb = 8;
            k_init_candidates<<<(n1 + wpb - 1) / wpb, 32 * wpb, 0, m->stream>>>(g2, s1.kps, s1.desc, n1, d_prev, window,
                                                                             st, cnt, out, fill);
        };
        rc = candidate_lists(m, n1, b, launch, start, count, keys, total);
        if (rc == ORBGPU_ERR_CAPACITY) {
            est = est + sizeof(uint64_t) * (size_t)total * 2;
            continue;
        }
        if (rc) return rc;
        int* matched_dist = b.take<int>(std::max(1, n2));
        int* m21 = b.take<int>(std::max(1, n2));
        int* m12 = b.take<int>(n1);
        int* bin_of = b.take<int>(n1);
        int* d_nm = b.take<int>(1);
        // F2's matched distances and matches in shared memory up to 6144
        // keypoints (48 KiB), else in the scratch buffers
        const int smem_n2 = n2 <= 6144 ? n2 : 0;
        k_init_resolve<<<1, 32, sizeof(int) * 2 * (size_t)smem_n2, m->stream>>>(
            s1.kps, n1, s2.kps, n2, start, count, keys, m->nnratio, m->check_ori, smem_n2, matched_dist, m21, m12,
            bin_of, d_nm);
        ORBGPU_CUDA_TRY(cudaGetLastError());
        ORBGPU_CUDA_TRY(cudaMemcpyAsync(matches12, m12, sizeof(int) * n1, cudaMemcpyDeviceToHost, m->stream));
        ORBGPU_CUDA_TRY(cudaMemcpyAsync(m->h_pinned, d_nm, sizeof(int), cudaMemcpyDeviceToHost, m->stream));
        ORBGPU_CUDA_TRY(cudaStreamSynchronize(m->stream));
        *nmatches = m->h_pinned[0];
        // vbPrevMatched update (src/ORBmatcher.cc:712-714)
        std::vector<orbgpu_keypoint> k2;
        if (f2->mem == ORBGPU_MEM_DEVICE) {
            k2.resize(n2);
            if (n2) ORBGPU_CUDA_TRY(cudaMemcpy(k2.data(), f2->keypoints, sizeof(orbgpu_keypoint) * n2, cudaMemcpyDeviceToHost));
        }
        const orbgpu_keypoint* K2 = f2->mem == ORBGPU_MEM_DEVICE ? k2.data() : f2->keypoints;
        for (int i1 = 0; i1 < n1; i1++)
            if (matches12[i1] >= 0) {
                prev_matched[2 * i1] = K2[matches12[i1]].x;
                prev_matched[2 * i1 + 1] = K2[matches12[i1]].y;
            }
        return ORBGPU_OK;
    }
    return ORBGPU_ERR_CAPACITY;
}

extern "C" int orbgpu_search_by_projection(orbgpu_matcher* m, const orbgpu_frame* f, const orbgpu_mappoint* mappoints,
                                           const uint8_t* mp_descriptors, int n_mappoints, float th,
                                           const uint8_t* claimed, int* match_out, int mem, int* nmatches) {
    if (!m || !frame_ok(f) || n_mappoints < 0 || (n_mappoints > 0 && (!mappoints || !mp_descriptors)) || !match_out ||
        !nmatches)
        return ORBGPU_ERR_BAD_ARG;
    const int n = f->n, M = n_mappoints;
    *nmatches = 0;
    size_t est = frame_stage_bytes(f) + grid_bytes(n) + (size_t)std::max(1, M) * (sizeof(orbgpu_mappoint) + 32 + 24) +
                 (size_t)n * 24 + 64 * 1024 + sizeof(uint64_t) * (size_t)std::max(1, M) * 64;
    for (int attempt = 0; attempt < 2; attempt++) {
        int rc = ensure_scratch(m, est);
        if (rc) return rc;
        Bump b{(uint8_t*)m->scratch, 0, m->scratch_bytes};
        Staged s;
        if ((rc = stage_frame(m, f, b, s))) return rc;
        GridDev g;
        if ((rc = build_grid(m, f, s, b, g))) return rc;
        const orbgpu_mappoint* d_mps = mappoints;
        const uint8_t* d_mpd = mp_descriptors;
        const uint8_t* d_claimed = claimed;
        int* d_match = match_out;
        if (mem != ORBGPU_MEM_DEVICE) {
            orbgpu_mappoint* a = b.take<orbgpu_mappoint>(std::max(1, M));
            uint8_t* dd = b.take<uint8_t>((size_t)std::max(1, M) * 32);
            if (M) {
                ORBGPU_CUDA_TRY(cudaMemcpyAsync(a, mappoints, sizeof(orbgpu_mappoint) * M, cudaMemcpyHostToDevice, m->stream));
                ORBGPU_CUDA_TRY(cudaMemcpyAsync(dd, mp_descriptors, 32 * (size_t)M, cudaMemcpyHostToDevice, m->stream));
            }
            d_mps = a;
            d_mpd = dd;
            if (claimed) {
                uint8_t* c = b.take<uint8_t>(std::max(1, n));
                if (n) ORBGPU_CUDA_TRY(cudaMemcpyAsync(c, claimed, n, cudaMemcpyHostToDevice, m->stream));
                d_claimed = c;
            }
            d_match = b.take<int>(std::max(1, n));
        }
        if (n > 0) k_init_match_out<<<(n + 255) / 256, 256, 0, m->stream>>>(d_claimed, n, d_match);
        int *start, *count, total = 0;
        uint64_t* keys = nullptr;
        auto launch = [&](const int* st, int* cnt, uint64_t* out, int fill) {
            const int wpb = 8;
            if (M > 0)
                k_proj_candidates<<<(M + wpb - 1) / wpb, 32 * wpb, 0, m->stream>>>(g, d_mps, d_mpd, M, th, m->nnratio, st,
                                                                                cnt, out, fill);
        };
        rc = candidate_lists(m, M, b, launch, start, count, keys, total);
        if (rc == ORBGPU_ERR_CAPACITY) {
            est = est + sizeof(uint64_t) * (size_t)total * 2;
            continue;
        }
        if (rc) return rc;
        int* d_nm = b.take<int>(1);
        int* claims3 = b.take<int>((size_t)3 * std::max(1, n));
        int* res = b.take<int>(std::max(1, M));
        int* changed = b.take<int>(PROJ_ROUNDS);
        ORBGPU_CUDA_TRY(cudaMemsetAsync(d_nm, 0, sizeof(int), m->stream));
        ORBGPU_CUDA_TRY(cudaMemsetAsync(claims3, 0x7f, sizeof(int) * (size_t)3 * std::max(1, n), m->stream));
        ORBGPU_CUDA_TRY(cudaMemsetAsync(res, 0xfe, sizeof(int) * std::max(1, M), m->stream));
        ORBGPU_CUDA_TRY(cudaMemsetAsync(changed, 0, sizeof(int) * PROJ_ROUNDS, m->stream));
        if (M > 0) {
            const int wpb = 8;
            const int warps = std::max(M, (n + 31) / 32);
            for (int r = 0; r < PROJ_ROUNDS; r++)
                k_proj_round<<<(warps + wpb - 1) / wpb, 32 * wpb, 0, m->stream>>>(g, M, start, count, keys, m->nnratio, r,
                                                                                claims3, res, changed, d_match);
            k_proj_finish<<<1, 256, 0, m->stream>>>(M, changed, res, d_match, d_nm);
            k_proj_resolve<<<1, 32, 0, m->stream>>>(g, M, start, count, keys, m->nnratio, d_match, d_nm, changed);
        }
        ORBGPU_CUDA_TRY(cudaGetLastError());
        if (mem != ORBGPU_MEM_DEVICE && n > 0)
            ORBGPU_CUDA_TRY(cudaMemcpyAsync(match_out, d_match, sizeof(int) * n, cudaMemcpyDeviceToHost, m->stream));
        ORBGPU_CUDA_TRY(cudaMemcpyAsync(m->h_pinned, d_nm, sizeof(int), cudaMemcpyDeviceToHost, m->stream));
        ORBGPU_CUDA_TRY(cudaStreamSynchronize(m->stream));
        *nmatches = m->h_pinned[0];
        return ORBGPU_OK;
    }
    return ORBGPU_ERR_CAPACITY;
}

// The reference's bForward / bBackward decision (src/ORBmatcher.cc:1724-1741):
// twc = -Rcw' tcw and tlc = Rlw twc + tlw with cv::Mat rounding (products
// accumulated in double, stored as float, then a float addition).
int orbgpu::motion_level_mode(const orbgpu_frame_motion& mo, int mono) {
    const float* T = mo.Tcw;
    const float tcw[3] = {T[3], T[7], T[11]};
    float twc[3];
    for (int r = 0; r < 3; r++) {
        const float col[3] = {-T[r], -T[4 + r], -T[8 + r]};
        double s = 0.0;
        for (int k = 0; k < 3; k++) s += (double)col[k] * (double)tcw[k];
        twc[r] = (float)s;
    }
    const float* L = mo.Tlw;
    double s = 0.0;
    for (int k = 0; k < 3; k++) s += (double)L[8 + k] * (double)twc[k];
    const float tlcz = (float)s + L[11];
    const bool fwd = tlcz > mo.b && !mono;
    const bool bwd = -tlcz > mo.b && !mono;
    return fwd ? 1 : bwd ? 2 : 0;
}

extern "C" int orbgpu_search_by_projection_frame(orbgpu_matcher* m, const orbgpu_frame* current,
                                                 const orbgpu_frame* last, const orbgpu_frame_mappoint* last_mappoints,
                                                 const uint8_t* last_mp_descriptors, const orbgpu_frame_motion* motion,
                                                 float th, int mono, const uint8_t* claimed, int* match_out, int mem,
                                                 int* nmatches) {
    if (!m || !frame_ok(current) || !last || last->n < 0 || last->n >= (1 << 20) || (last->n > 0 && !last->keypoints) ||
        !motion || !match_out || !nmatches || (last->n > 0 && (!last_mappoints || !last_mp_descriptors)))
        return ORBGPU_ERR_BAD_ARG;
    const int n = current->n, M = last->n;
    *nmatches = 0;
    const int mode = motion_level_mode(*motion, mono);
    FrameMotionDev mo;
    std::memcpy(mo.T, motion->Tcw, sizeof(mo.T));
    mo.fx = motion->fx;
    mo.fy = motion->fy;
    mo.cx = motion->cx;
    mo.cy = motion->cy;
    mo.bf = motion->bf;
    mo.maxX = (float)current->width;
    mo.maxY = (float)current->height;
    mo.level_mode = mode;
    size_t est = frame_stage_bytes(current) + grid_bytes(n) +
                 (size_t)std::max(1, M) * (sizeof(orbgpu_frame_mappoint) + sizeof(orbgpu_keypoint) + 32 + 32) +
                 (size_t)std::max(1, n) * 32 + 64 * 1024 + sizeof(uint64_t) * (size_t)std::max(1, M) * 32;
    for (int attempt = 0; attempt < 2; attempt++) {
        int rc = ensure_scratch(m, est);
        if (rc) return rc;
        Bump b{(uint8_t*)m->scratch, 0, m->scratch_bytes};
        Staged s;
        if ((rc = stage_frame(m, current, b, s))) return rc;
        GridDev g;
        if ((rc = build_grid(m, current, s, b, g))) return rc;
        const orbgpu_keypoint* d_lk = last->keypoints;
        if (last->mem != ORBGPU_MEM_DEVICE) {
            orbgpu_keypoint* k = b.take<orbgpu_keypoint>(std::max(1, M));
            if (M)
                ORBGPU_CUDA_TRY(cudaMemcpyAsync(k, last->keypoints, sizeof(orbgpu_keypoint) * M, cudaMemcpyHostToDevice,
                                                m->stream));
            d_lk = k;
        }
        const orbgpu_frame_mappoint* d_mps = last_mappoints;
        const uint8_t* d_mpd = last_mp_descriptors;
        const uint8_t* d_claimed = claimed;
        int* d_match = match_out;
        if (mem != ORBGPU_MEM_DEVICE) {
            orbgpu_frame_mappoint* a = b.take<orbgpu_frame_mappoint>(std::max(1, M));
            uint8_t* dd = b.take<uint8_t>((size_t)std::max(1, M) * 32);
            if (M) {
                ORBGPU_CUDA_TRY(cudaMemcpyAsync(a, last_mappoints, sizeof(orbgpu_frame_mappoint) * M,
                                                cudaMemcpyHostToDevice, m->stream));
                ORBGPU_CUDA_TRY(cudaMemcpyAsync(dd, last_mp_descriptors, 32 * (size_t)M, cudaMemcpyHostToDevice,
                                                m->stream));
            }
            d_mps = a;
            d_mpd = dd;
            if (claimed) {
                uint8_t* c = b.take<uint8_t>(std::max(1, n));
                if (n) ORBGPU_CUDA_TRY(cudaMemcpyAsync(c, claimed, n, cudaMemcpyHostToDevice, m->stream));
                d_claimed = c;
            }
            d_match = b.take<int>(std::max(1, n));
        }
        if (n > 0) k_init_match_out<<<(n + 255) / 256, 256, 0, m->stream>>>(d_claimed, n, d_match);
        int *start, *count, total = 0;
        uint64_t* keys = nullptr;
        auto launch = [&](const int* st, int* cnt, uint64_t* out, int fill) {
            const int wpb = 8;
            if (M > 0)
                k_pf_candidates<<<(M + wpb - 1) / wpb, 32 * wpb, 0, m->stream>>>(g, mo, d_lk, d_mps, d_mpd, M, th, st,
                                                                              cnt, out, fill);
        };
        rc = candidate_lists(m, M, b, launch, start, count, keys, total);
        if (rc == ORBGPU_ERR_CAPACITY) {
            est = est + sizeof(uint64_t) * (size_t)total * 2;
            continue;
        }
        if (rc) return rc;
        int* d_nm = b.take<int>(1);
        int* claims3 = b.take<int>((size_t)3 * std::max(1, n));
        int* res = b.take<int>(std::max(1, M));
        int* changed = b.take<int>(PROJ_ROUNDS);
        int* owner = b.take<int>(std::max(1, n));
        int* nulled = b.take<int>(std::max(1, n));
        int* bin_of = b.take<int>(std::max(1, M));
        ORBGPU_CUDA_TRY(cudaMemsetAsync(d_nm, 0, sizeof(int), m->stream));
        ORBGPU_CUDA_TRY(cudaMemsetAsync(claims3, 0x7f, sizeof(int) * (size_t)3 * std::max(1, n), m->stream));
        ORBGPU_CUDA_TRY(cudaMemsetAsync(res, 0xfe, sizeof(int) * std::max(1, M), m->stream));
        ORBGPU_CUDA_TRY(cudaMemsetAsync(changed, 0, sizeof(int) * PROJ_ROUNDS, m->stream));
        if (M > 0 && n > 0) {
            const int wpb = 8;
            const int warps = std::max(M, (n + 31) / 32);
            for (int r = 0; r < PROJ_ROUNDS; r++)
                k_pf_round<<<(warps + wpb - 1) / wpb, 32 * wpb, 0, m->stream>>>(n, M, start, count, keys, d_mps, r,
                                                                              claims3, res, changed, d_match);
            k_pf_serial<<<1, 32, 0, m->stream>>>(n, M, start, count, keys, d_mps, changed, res, claims3, d_match);
            k_pf_finish<<<1, 1024, 0, m->stream>>>(n, M, res, d_lk, s.kps, m->check_ori, owner, bin_of, nulled, d_match,
                                                   d_nm);
        }
        ORBGPU_CUDA_TRY(cudaGetLastError());
        if (mem != ORBGPU_MEM_DEVICE && n > 0)
            ORBGPU_CUDA_TRY(cudaMemcpyAsync(match_out, d_match, sizeof(int) * n, cudaMemcpyDeviceToHost, m->stream));
        ORBGPU_CUDA_TRY(cudaMemcpyAsync(m->h_pinned, d_nm, sizeof(int), cudaMemcpyDeviceToHost, m->stream));
        ORBGPU_CUDA_TRY(cudaStreamSynchronize(m->stream));
        *nmatches = m->h_pinned[0];
        return ORBGPU_OK;
    }
    return ORBGPU_ERR_CAPACITY;
}

static int search_projection_keyframe(orbgpu_matcher* m, const orbgpu_frame* current, const KeyframeProjDev& kp,
                                      const orbgpu_keypoint* kf_keypoints, const orbgpu_mappoint_geometry* mappoints,
                                      const uint8_t* mp_descriptors, const uint8_t* usable, int n_kf, float th,
                                      const uint8_t* claimed, int* match_out, int mem, int* nmatches);

extern "C" int orbgpu_search_by_projection_keyframe(orbgpu_matcher* m, const orbgpu_frame* current,
                                                    const orbgpu_frustum_frame* pose,
                                                    const orbgpu_keypoint* kf_keypoints,
                                                    const orbgpu_mappoint_geometry* mappoints,
                                                    const uint8_t* mp_descriptors, const uint8_t* usable, int n_kf,
                                                    float th, int orbdist, const uint8_t* claimed, int* match_out,
                                                    int mem, int* nmatches) {
    if (!m || !frame_ok(current) || !pose || n_kf < 0 || n_kf >= (1 << 20) || !match_out || !nmatches ||
        (n_kf > 0 && (!kf_keypoints || !mappoints || !mp_descriptors || !usable)) || pose->nlevels < 1 ||
        pose->nlevels > 16)
        return ORBGPU_ERR_BAD_ARG;
    KeyframeProjDev kp;
    std::memset(&kp, 0, sizeof(kp));
    for (int r = 0; r < 3; r++) {
        for (int c = 0; c < 3; c++) kp.T[4 * r + c] = pose->Rcw[3 * r + c];
        kp.T[4 * r + 3] = pose->tcw[r];
        kp.Ow[r] = pose->Ow[r];
    }
    kp.fx = pose->fx;
    kp.fy = pose->fy;
    kp.cx = pose->cx;
    kp.cy = pose->cy;
    kp.maxX = (float)current->width;
    kp.maxY = (float)current->height;
    kp.nlevels = pose->nlevels;
    std::memcpy(kp.level_above, pose->level_above, sizeof(kp.level_above));
    kp.orbdist = orbdist;
    kp.sim3 = 0;
    return search_projection_keyframe(m, current, kp, kf_keypoints, mappoints, mp_descriptors, usable, n_kf, th,
                                      claimed, match_out, mem, nmatches);
}

// The candidate lists and in-order resolution shared by the relocalisation
// and the loop-closing projection searches.
static int search_projection_keyframe(orbgpu_matcher* m, const orbgpu_frame* current, const KeyframeProjDev& kp,
                                      const orbgpu_keypoint* kf_keypoints, const orbgpu_mappoint_geometry* mappoints,
                                      const uint8_t* mp_descriptors, const uint8_t* usable, int n_kf, float th,
                                      const uint8_t* claimed, int* match_out, int mem, int* nmatches) {
    const int n = current->n, M = n_kf;
    *nmatches = 0;
    size_t est = frame_stage_bytes(current) + grid_bytes(n) +
                 (size_t)std::max(1, M) * (sizeof(orbgpu_mappoint_geometry) + sizeof(orbgpu_keypoint) + 32 + 1 + 32) +
                 (size_t)std::max(1, n) * 32 + 64 * 1024 + sizeof(uint64_t) * (size_t)std::max(1, M) * 32;
    for (int attempt = 0; attempt < 2; attempt++) {
        int rc = ensure_scratch(m, est);
        if (rc) return rc;
        Bump b{(uint8_t*)m->scratch, 0, m->scratch_bytes};
        Staged s;
        if ((rc = stage_frame(m, current, b, s))) return rc;
        GridDev g;
        if ((rc = build_grid(m, current, s, b, g))) return rc;
        const orbgpu_keypoint* d_kk = kf_keypoints;
        const orbgpu_mappoint_geometry* d_mps = mappoints;
        const uint8_t* d_mpd = mp_descriptors;
        const uint8_t* d_use = usable;
        const uint8_t* d_claimed = claimed;
        int* d_match = match_out;
        if (mem != ORBGPU_MEM_DEVICE) {
            orbgpu_keypoint* k = b.take<orbgpu_keypoint>(std::max(1, M));
            orbgpu_mappoint_geometry* a = b.take<orbgpu_mappoint_geometry>(std::max(1, M));
            uint8_t* dd = b.take<uint8_t>((size_t)std::max(1, M) * 32);
            uint8_t* uu = b.take<uint8_t>(std::max(1, M));
            if (M) {
                if (kf_keypoints)
                    ORBGPU_CUDA_TRY(cudaMemcpyAsync(k, kf_keypoints, sizeof(orbgpu_keypoint) * M,
                                                    cudaMemcpyHostToDevice, m->stream));
                ORBGPU_CUDA_TRY(cudaMemcpyAsync(a, mappoints, sizeof(orbgpu_mappoint_geometry) * M,
                                                cudaMemcpyHostToDevice, m->stream));
                ORBGPU_CUDA_TRY(cudaMemcpyAsync(dd, mp_descriptors, 32 * (size_t)M, cudaMemcpyHostToDevice,
                                                m->stream));
                ORBGPU_CUDA_TRY(cudaMemcpyAsync(uu, usable, M, cudaMemcpyHostToDevice, m->stream));
            }
            d_kk = k;
            d_mps = a;
            d_mpd = dd;
            d_use = uu;
            if (claimed) {
                uint8_t* c = b.take<uint8_t>(std::max(1, n));
                if (n) ORBGPU_CUDA_TRY(cudaMemcpyAsync(c, claimed, n, cudaMemcpyHostToDevice, m->stream));
                d_claimed = c;
            }
            d_match = b.take<int>(std::max(1, n));
        }
        if (n > 0) k_init_match_out<<<(n + 255) / 256, 256, 0, m->stream>>>(d_claimed, n, d_match);
        int *start, *count, total = 0;
        uint64_t* keys = nullptr;
        auto launch = [&](const int* st, int* cnt, uint64_t* out, int fill) {
            const int wpb = 8;
            if (M > 0)
                k_pkf_candidates<<<(M + wpb - 1) / wpb, 32 * wpb, 0, m->stream>>>(g, kp, d_mps, d_use, d_mpd, M, th,
                                                                               st, cnt, out, fill);
        };
        rc = candidate_lists(m, M, b, launch, start, count, keys, total);
        if (rc == ORBGPU_ERR_CAPACITY) {
            est = est + sizeof(uint64_t) * (size_t)total * 2;
            continue;
        }
        if (rc) return rc;
        int* d_nm = b.take<int>(1);
        int* claims3 = b.take<int>((size_t)3 * std::max(1, n));
        int* res = b.take<int>(std::max(1, M));
        int* changed = b.take<int>(PROJ_ROUNDS);
        int* owner = b.take<int>(std::max(1, n));
        int* nulled = b.take<int>(std::max(1, n));
        int* bin_of = b.take<int>(std::max(1, M));
        ORBGPU_CUDA_TRY(cudaMemsetAsync(d_nm, 0, sizeof(int), m->stream));
        ORBGPU_CUDA_TRY(cudaMemsetAsync(claims3, 0x7f, sizeof(int) * (size_t)3 * std::max(1, n), m->stream));
        ORBGPU_CUDA_TRY(cudaMemsetAsync(res, 0xfe, sizeof(int) * std::max(1, M), m->stream));
        ORBGPU_CUDA_TRY(cudaMemsetAsync(changed, 0, sizeof(int) * PROJ_ROUNDS, m->stream));
        if (M > 0 && n > 0) {
            const int wpb = 8;
            const int warps = std::max(M, (n + 31) / 32);
            // every assignment blocks (src/ORBmatcher.cc:1951: any map point on the keypoint)
            for (int r = 0; r < PROJ_ROUNDS; r++)
                k_pf_round<<<(warps + wpb - 1) / wpb, 32 * wpb, 0, m->stream>>>(n, M, start, count, keys, nullptr, r,
                                                                              claims3, res, changed, d_match);
            k_pf_serial<<<1, 32, 0, m->stream>>>(n, M, start, count, keys, nullptr, changed, res, claims3, d_match);
            // the loop-closing search has no rotation check
            k_pf_finish<<<1, 1024, 0, m->stream>>>(n, M, res, d_kk, s.kps, kp.sim3 ? 0 : m->check_ori, owner, bin_of,
                                                   nulled, d_match, d_nm);
        }
        ORBGPU_CUDA_TRY(cudaGetLastError());
        if (mem != ORBGPU_MEM_DEVICE && n > 0)
            ORBGPU_CUDA_TRY(cudaMemcpyAsync(match_out, d_match, sizeof(int) * n, cudaMemcpyDeviceToHost, m->stream));
        ORBGPU_CUDA_TRY(cudaMemcpyAsync(m->h_pinned, d_nm, sizeof(int), cudaMemcpyDeviceToHost, m->stream));
        ORBGPU_CUDA_TRY(cudaStreamSynchronize(m->stream));
        *nmatches = m->h_pinned[0];
        return ORBGPU_OK;
    }
    return ORBGPU_ERR_CAPACITY;
}

extern "C" int orbgpu_search_by_projection_sim3(orbgpu_matcher* m, const orbgpu_frame* keyframe, const float* Scw,
                                                float fx, float fy, float cx, float cy, float scale_factor,
                                                int nlevels, const orbgpu_mappoint_geometry* points,
                                                const uint8_t* point_descriptors, const uint8_t* usable, int npoints,
                                                int th, const uint8_t* matched, int* match_out, int mem,
                                                int* nmatches) {
    if (!m || !frame_ok(keyframe) || !Scw || npoints < 0 || npoints >= (1 << 20) || !match_out || !nmatches ||
        (npoints > 0 && (!points || !point_descriptors || !usable)) || nlevels < 1 || nlevels > 16 ||
        !(scale_factor > 1.0f))
        return ORBGPU_ERR_BAD_ARG;
    // Scw = [s R | s t]: s = sqrt(row 0 . row 0) (a double dot product, the
    // root rounded to float), R and t divided by it as floats, Ow = -R^T t
    // (src/ORBmatcher.cc:436-442)
    double d = 0.0;
    for (int k = 0; k < 3; k++) d += (double)Scw[k] * (double)Scw[k];
    const float scw = (float)std::sqrt(d);
    KeyframeProjDev kp;
    std::memset(&kp, 0, sizeof(kp));
    for (int r = 0; r < 3; r++)
        for (int c = 0; c < 4; c++) kp.T[4 * r + c] = Scw[4 * r + c] / scw;
    for (int i = 0; i < 3; i++) {
        double s = 0.0;
        for (int k = 0; k < 3; k++) s += (double)(-kp.T[4 * k + i]) * (double)kp.T[4 * k + 3];
        kp.Ow[i] = (float)s;
    }
    kp.fx = fx;
    kp.fy = fy;
    kp.cx = cx;
    kp.cy = cy;
    kp.maxX = (float)keyframe->width;
    kp.maxY = (float)keyframe->height;
    // MapPoint::PredictScale(dist, KeyFrame*): the thresholds of the frame version
    orbgpu_frustum_frame tmp;
    const float eye[12] = {1, 0, 0, 0, 0, 1, 0, 0, 0, 0, 1, 0};
    int rc = orbgpu_frustum_frame_init(eye, fx, fy, cx, cy, 0, 0, 1, 0, 1, scale_factor, nlevels, &tmp);
    if (rc) return rc;
    kp.nlevels = nlevels;
    std::memcpy(kp.level_above, tmp.level_above, sizeof(kp.level_above));
    kp.orbdist = ORBGPU_TH_LOW;
    kp.sim3 = 1;
    return search_projection_keyframe(m, keyframe, kp, nullptr, points, point_descriptors, usable, npoints, (float)th,
                                      matched, match_out, mem, nmatches);
}

// Fuse's choice per map point: the first least distance of its candidates
// (candidates are already cut at TH_LOW), with no interaction between map
// points -- the map updates it leads to are applied in order by the caller.
__global__ void k_fuse_pick(int m, const int* cand_start, const int* cand_count, const uint64_t* cands,
                            int* target, int* dist_out) {
    const int lane = threadIdx.x & 31;
    const int i = blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5);
    if (i >= m) return;
    uint64_t best = ~0ull;
    for (int b = lane; b < cand_count[i]; b += 32) {
        const uint64_t key = cands[cand_start[i] + b];
        best = key < best ? key : best;
    }
    for (int o = 16; o > 0; o >>= 1) {
        const uint64_t ob = __shfl_xor_sync(0xffffffffu, best, o);
        best = ob < best ? ob : best;
    }
    if (lane == 0) {
        target[i] = best == ~0ull ? -1 : (int)(best & 0xFFFFF);
        if (dist_out) dist_out[i] = best == ~0ull ? 256 : (int)(best >> 40);
    }
}

static int fuse_pick_run(orbgpu_matcher* m, const orbgpu_frame* keyframe, const KeyframeProjDev& kp,
                         const orbgpu_mappoint_geometry* mappoints, const uint8_t* mp_descriptors,
                         const uint8_t* usable, int n_mp, float th, int* target, int* dist, int mem);

extern "C" int orbgpu_fuse_candidates(orbgpu_matcher* m, const orbgpu_frame* keyframe, const float* Tcw, float fx,
                                      float fy, float cx, float cy, float bf, float scale_factor, int nlevels,
                                      const float* inv_level_sigma2, const orbgpu_mappoint_geometry* mappoints,
                                      const uint8_t* mp_descriptors, const uint8_t* usable, int n_mp, float th,
                                      int* target, int* dist, int mem) {
    if (!m || !frame_ok(keyframe) || !Tcw || !inv_level_sigma2 || n_mp < 0 || n_mp >= (1 << 20) || !target ||
        (n_mp > 0 && (!mappoints || !mp_descriptors || !usable)) || nlevels < 1 || nlevels > 16 ||
        !(scale_factor > 1.0f))
        return ORBGPU_ERR_BAD_ARG;
    KeyframeProjDev kp;
    std::memset(&kp, 0, sizeof(kp));
    std::memcpy(kp.T, Tcw, sizeof(kp.T));
    // Ow = GetCameraCenter() = -Rcw^T tcw
    for (int i = 0; i < 3; i++) {
        double s = 0.0;
        for (int k = 0; k < 3; k++) s += (double)(-Tcw[4 * k + i]) * (double)Tcw[4 * k + 3];
        kp.Ow[i] = (float)s;
    }
    kp.fx = fx;
    kp.fy = fy;
    kp.cx = cx;
    kp.cy = cy;
    kp.bf = bf;
    kp.maxX = (float)keyframe->width;
    kp.maxY = (float)keyframe->height;
    orbgpu_frustum_frame tmp;
    const float eye[12] = {1, 0, 0, 0, 0, 1, 0, 0, 0, 0, 1, 0};
    int rc = orbgpu_frustum_frame_init(eye, fx, fy, cx, cy, 0, 0, 1, 0, 1, scale_factor, nlevels, &tmp);
    if (rc) return rc;
    kp.nlevels = nlevels;
    std::memcpy(kp.level_above, tmp.level_above, sizeof(kp.level_above));
    for (int l = 0; l < nlevels; l++) kp.inv_sigma2[l] = inv_level_sigma2[l];
    kp.orbdist = ORBGPU_TH_LOW;
    kp.sim3 = 1;
    kp.fuse = 1;
    return fuse_pick_run(m, keyframe, kp, mappoints, mp_descriptors, usable, n_mp, th, target, dist, mem);
}

// The candidate lists of a fuse search and the choice of every map point.
static int fuse_pick_run(orbgpu_matcher* m, const orbgpu_frame* keyframe, const KeyframeProjDev& kp,
                         const orbgpu_mappoint_geometry* mappoints, const uint8_t* mp_descriptors,
                         const uint8_t* usable, int n_mp, float th, int* target, int* dist, int mem) {
    int rc;
    const int n = keyframe->n, M = n_mp;
    size_t est = frame_stage_bytes(keyframe) + grid_bytes(n) +
                 (size_t)std::max(1, M) * (sizeof(orbgpu_mappoint_geometry) + 32 + 1 + 2 * sizeof(int) + 32) +
                 64 * 1024 + sizeof(uint64_t) * (size_t)std::max(1, M) * 32;
    for (int attempt = 0; attempt < 2; attempt++) {
        rc = ensure_scratch(m, est);
        if (rc) return rc;
        Bump b{(uint8_t*)m->scratch, 0, m->scratch_bytes};
        Staged s;
        if ((rc = stage_frame(m, keyframe, b, s))) return rc;
        GridDev g;
        if ((rc = build_grid(m, keyframe, s, b, g))) return rc;
        const orbgpu_mappoint_geometry* d_mps = mappoints;
        const uint8_t* d_mpd = mp_descriptors;
        const uint8_t* d_use = usable;
        int* d_t = target;
        int* d_d = dist;
        if (mem != ORBGPU_MEM_DEVICE) {
            orbgpu_mappoint_geometry* a = b.take<orbgpu_mappoint_geometry>(std::max(1, M));
            uint8_t* dd = b.take<uint8_t>((size_t)std::max(1, M) * 32);
            uint8_t* uu = b.take<uint8_t>(std::max(1, M));
            if (M) {
                ORBGPU_CUDA_TRY(cudaMemcpyAsync(a, mappoints, sizeof(orbgpu_mappoint_geometry) * M,
                                                cudaMemcpyHostToDevice, m->stream));
                ORBGPU_CUDA_TRY(cudaMemcpyAsync(dd, mp_descriptors, 32 * (size_t)M, cudaMemcpyHostToDevice,
                                                m->stream));
                ORBGPU_CUDA_TRY(cudaMemcpyAsync(uu, usable, M, cudaMemcpyHostToDevice, m->stream));
            }
            d_mps = a;
            d_mpd = dd;
            d_use = uu;
            d_t = b.take<int>(std::max(1, M));
            d_d = dist ? b.take<int>(std::max(1, M)) : nullptr;
        }
        int *start, *count, total = 0;
        uint64_t* keys = nullptr;
        auto launch = [&](const int* st, int* cnt, uint64_t* out, int fill) {
            const int wpb = 8;
            if (M > 0)
                k_pkf_candidates<<<(M + wpb - 1) / wpb, 32 * wpb, 0, m->stream>>>(g, kp, d_mps, d_use, d_mpd, M, th,
                                                                               st, cnt, out, fill);
        };
        rc = candidate_lists(m, M, b, launch, start, count, keys, total);
        if (rc == ORBGPU_ERR_CAPACITY) {
            est = est + sizeof(uint64_t) * (size_t)total * 2;
            continue;
        }
        if (rc) return rc;
        if (M > 0) k_fuse_pick<<<(M + 7) / 8, 256, 0, m->stream>>>(M, start, count, keys, d_t, d_d);
        ORBGPU_CUDA_TRY(cudaGetLastError());
        if (mem != ORBGPU_MEM_DEVICE && M > 0) {
            ORBGPU_CUDA_TRY(cudaMemcpyAsync(target, d_t, sizeof(int) * M, cudaMemcpyDeviceToHost, m->stream));
            if (dist) ORBGPU_CUDA_TRY(cudaMemcpyAsync(dist, d_d, sizeof(int) * M, cudaMemcpyDeviceToHost, m->stream));
        }
        ORBGPU_CUDA_TRY(cudaStreamSynchronize(m->stream));
        return ORBGPU_OK;
    }
    return ORBGPU_ERR_CAPACITY;
}

extern "C" int orbgpu_fuse_sim3_candidates(orbgpu_matcher* m, const orbgpu_frame* keyframe, const float* Scw,
                                           float fx, float fy, float cx, float cy, float scale_factor, int nlevels,
                                           const orbgpu_mappoint_geometry* points, const uint8_t* point_descriptors,
                                           const uint8_t* usable, int npoints, float th, int* target, int* dist,
                                           int mem) {
    if (!m || !frame_ok(keyframe) || !Scw || npoints < 0 || npoints >= (1 << 20) || !target ||
        (npoints > 0 && (!points || !point_descriptors || !usable)) || nlevels < 1 || nlevels > 16 ||
        !(scale_factor > 1.0f))
        return ORBGPU_ERR_BAD_ARG;
    // the Sim3 de-scaled as in SearchByProjection(KeyFrame*, Scw, ...)
    double d = 0.0;
    for (int k = 0; k < 3; k++) d += (double)Scw[k] * (double)Scw[k];
    const float scw = (float)std::sqrt(d);
    KeyframeProjDev kp;
    std::memset(&kp, 0, sizeof(kp));
    for (int r = 0; r < 3; r++)
        for (int c = 0; c < 4; c++) kp.T[4 * r + c] = Scw[4 * r + c] / scw;
    for (int i = 0; i < 3; i++) {
        double s = 0.0;
        for (int k = 0; k < 3; k++) s += (double)(-kp.T[4 * k + i]) * (double)kp.T[4 * k + 3];
        kp.Ow[i] = (float)s;
    }
    kp.fx = fx;
    kp.fy = fy;
    kp.cx = cx;
    kp.cy = cy;
    kp.maxX = (float)keyframe->width;
    kp.maxY = (float)keyframe->height;
    orbgpu_frustum_frame tmp;
    const float eye[12] = {1, 0, 0, 0, 0, 1, 0, 0, 0, 0, 1, 0};
    int rc = orbgpu_frustum_frame_init(eye, fx, fy, cx, cy, 0, 0, 1, 0, 1, scale_factor, nlevels, &tmp);
    if (rc) return rc;
    kp.nlevels = nlevels;
    std::memcpy(kp.level_above, tmp.level_above, sizeof(kp.level_above));
    kp.orbdist = ORBGPU_TH_LOW;
    kp.sim3 = 1;
    kp.invz_double = 1;
    return fuse_pick_run(m, keyframe, kp, points, point_descriptors, usable, npoints, th, target, dist, mem);
}

// SearchBySim3's geometry: cv::Mat products accumulated in double and
// rounded to float (plus a float add), scalar products of float matrices as
// float products of the scalar rounded to float.
static void mat3_times(const float* A, const float* x, float* out) {
    for (int r = 0; r < 3; r++) {
        double s = 0.0;
        for (int k = 0; k < 3; k++) s += (double)A[3 * r + k] * (double)x[k];
        out[r] = (float)s;
    }
}

extern "C" int orbgpu_search_by_sim3(orbgpu_matcher* m, const orbgpu_frame* kf1, const orbgpu_frame* kf2,
                                     const float* T1w, const float* T2w, float s12, const float* R12,
                                     const float* t12, float fx, float fy, float cx, float cy, float scale_factor,
                                     int nlevels, const orbgpu_mappoint_geometry* mps1, const uint8_t* mpd1,
                                     const uint8_t* usable1, const orbgpu_mappoint_geometry* mps2,
                                     const uint8_t* mpd2, const uint8_t* usable2, float th, int* match12,
                                     int* nfound) {
    if (!m || !frame_ok(kf1) || !frame_ok(kf2) || !T1w || !T2w || !R12 || !t12 || !match12 || !nfound ||
        nlevels < 1 || nlevels > 16 || !(scale_factor > 1.0f) || kf1->n < 0 || kf2->n < 0 ||
        (kf1->n > 0 && (!mps1 || !mpd1 || !usable1)) || (kf2->n > 0 && (!mps2 || !mpd2 || !usable2)))
        return ORBGPU_ERR_BAD_ARG;
    const int N1 = kf1->n, N2 = kf2->n;
    // sR12 = s12 * R12, sR21 = (1.0 / s12) * R12^T, t21 = -sR21 * t12
    // (src/ORBmatcher.cc:1456-1463)
    const float inv_s = (float)(1.0 / (double)s12);
    float sR12[9], sR21[9], nsR21[9], t21[3];
    for (int r = 0; r < 3; r++)
        for (int c = 0; c < 3; c++) {
            sR12[3 * r + c] = R12[3 * r + c] * s12;
            sR21[3 * r + c] = R12[3 * c + r] * inv_s;
            nsR21[3 * r + c] = -sR21[3 * r + c];
        }
    mat3_times(nsR21, t12, t21);
    orbgpu_frustum_frame tmp;
    const float eye[12] = {1, 0, 0, 0, 0, 1, 0, 0, 0, 0, 1, 0};
    int rc = orbgpu_frustum_frame_init(eye, fx, fy, cx, cy, 0, 0, 1, 0, 1, scale_factor, nlevels, &tmp);
    if (rc) return rc;
    auto pass = [&](const orbgpu_frame* target_kf, const float* Tw, const float* sR, const float* t,
                    const orbgpu_mappoint_geometry* mps, const uint8_t* mpd, const uint8_t* use, int n,
                    std::vector<int>& out) {
        KeyframeProjDev kp;
        std::memset(&kp, 0, sizeof(kp));
        std::memcpy(kp.T, Tw, sizeof(kp.T));
        for (int r = 0; r < 3; r++) {
            for (int c = 0; c < 3; c++) kp.T2[4 * r + c] = sR[3 * r + c];
            kp.T2[4 * r + 3] = t[r];
        }
        kp.fx = fx;
        kp.fy = fy;
        kp.cx = cx;
        kp.cy = cy;
        kp.maxX = (float)target_kf->width;
        kp.maxY = (float)target_kf->height;
        kp.nlevels = nlevels;
        std::memcpy(kp.level_above, tmp.level_above, sizeof(kp.level_above));
        kp.orbdist = ORBGPU_TH_HIGH;
        kp.sim3 = 1;
        kp.invz_double = 1;
        kp.chain = 1;
        out.assign(std::max(n, 1), -1);
        return fuse_pick_run(m, target_kf, kp, mps, mpd, use, n, th, out.data(), nullptr, ORBGPU_MEM_HOST);
    };
    // vnMatch1: pKF1's map points into pKF2; vnMatch2: pKF2's into pKF1
    std::vector<int> match1, match2;
    if ((rc = pass(kf2, T1w, sR21, t21, mps1, mpd1, usable1, N1, match1))) return rc;
    if ((rc = pass(kf1, T2w, sR12, t12, mps2, mpd2, usable2, N2, match2))) return rc;
    int found = 0;
    for (int i1 = 0; i1 < N1; i1++) {
        const int i2 = match1[i1];
        match12[i1] = (i2 >= 0 && i2 < N2 && match2[i2] == i1) ? i2 : -1;
        found += match12[i1] >= 0;
    }
    *nfound = found;
    return ORBGPU_OK;
}

extern "C" int orbgpu_compute_stereo_matches(orbgpu_matcher* m, const orbgpu_extractor* left,
                                             const orbgpu_extractor* right, const orbgpu_frame* fl,
                                             const orbgpu_frame* fr, float bf, float fx, float* uright, float* depth,
                                             int mem) {
    if (!m || !left || !right || !frame_ok(fl) || !frame_ok(fr) || !uright || !depth) return ORBGPU_ERR_BAD_ARG;
    const int nL = fl->n, nR = fr->n;
    if (nL == 0) return ORBGPU_OK;
    StereoLevels lv;
    std::memset(&lv, 0, sizeof(lv));
    int nlev = fl->nlevels;
    for (int l = 0; l < nlev; l++) {
        const uint8_t *pl, *pr;
        int w, h, w2, h2;
        size_t pitch, pitch2;
        if (orbgpu_extractor_pyramid_level(left, l, &pl, &w, &h, &pitch) ||
            orbgpu_extractor_pyramid_level(right, l, &pr, &w2, &h2, &pitch2) || w != w2 || h != h2 || pitch != pitch2)
            return ORBGPU_ERR_BAD_ARG;
        lv.left[l] = pl;
        lv.right[l] = pr;
        lv.w[l] = w;
        lv.h[l] = h;
        lv.pitch[l] = (int)pitch;
        lv.scale[l] = fl->scale_factors[l];
        lv.inv_scale[l] = 1.0f / fl->scale_factors[l];
    }
    lv.nlevels = nlev;
    const int nRows = lv.h[0];
    float maxscale = 1.0f;
    for (int l = 0; l < nlev; l++) maxscale = std::max(maxscale, lv.scale[l]);
    const int rows_per_key = 2 * (int)std::ceil(2.0f * maxscale) + 4;
    int sort_cap = 1;
    while (sort_cap < nL) sort_cap <<= 1;
    const size_t est = frame_stage_bytes(fl) + frame_stage_bytes(fr) + (size_t)(2 * nRows + 8) * sizeof(int) +
                       (size_t)nR * rows_per_key * sizeof(int) + (size_t)nL * 3 * sizeof(float) + sort_cap * sizeof(int) +
                       64 * 1024;
    int rc = ensure_scratch(m, est);
    if (rc) return rc;
    Bump b{(uint8_t*)m->scratch, 0, m->scratch_bytes};
    Staged sl, sr;
    if ((rc = stage_frame(m, fl, b, sl)) || (rc = stage_frame(m, fr, b, sr))) return rc;
    int* row_count = b.take<int>(nRows + 1);
    int* row_start = b.take<int>(nRows + 1);
    int* cursor = b.take<int>(nRows + 1);
    int* row_keys = b.take<int>((size_t)std::max(1, nR) * rows_per_key);
    int* d_total = b.take<int>(1);
    float* d_ur = uright;
    float* d_dp = depth;
    if (mem != ORBGPU_MEM_DEVICE) {
        d_ur = b.take<float>(nL);
        d_dp = b.take<float>(nL);
    }
    int* sad = b.take<int>(nL);
    int* sort_buf = b.take<int>(sort_cap);
    int* status = b.take<int>(2);
    ORBGPU_CUDA_TRY(cudaMemsetAsync(row_count, 0, sizeof(int) * (nRows + 1), m->stream));
    ORBGPU_CUDA_TRY(cudaMemsetAsync(status, 0, sizeof(int) * 2, m->stream));
    if (nR > 0) k_stereo_rows_count<<<(nR + 255) / 256, 256, 0, m->stream>>>(sr.kps, nR, lv, nRows, row_count);
    k_exclusive_scan<<<1, 1024, 0, m->stream>>>(row_count, nRows + 1, row_start, d_total);
    ORBGPU_CUDA_TRY(cudaMemcpyAsync(cursor, row_start, sizeof(int) * (nRows + 1), cudaMemcpyDeviceToDevice, m->stream));
    if (nR > 0) k_stereo_rows_fill<<<(nR + 255) / 256, 256, 0, m->stream>>>(sr.kps, nR, lv, nRows, cursor, row_keys);
    const int wpb = 8;
    k_stereo_match<<<(nL + wpb - 1) / wpb, 32 * wpb, 0, m->stream>>>(sl.kps, sl.desc, nL, sr.kps, sr.desc, lv, nRows,
                                                                   row_start, row_keys, bf, fx, d_ur, d_dp, sad, status);
    k_stereo_median<<<1, 1024, 0, m->stream>>>(nL, sad, d_ur, d_dp, sort_buf, sort_cap, status + 1);
    ORBGPU_CUDA_TRY(cudaGetLastError());
    if (mem != ORBGPU_MEM_DEVICE) {
        ORBGPU_CUDA_TRY(cudaMemcpyAsync(uright, d_ur, sizeof(float) * nL, cudaMemcpyDeviceToHost, m->stream));
        ORBGPU_CUDA_TRY(cudaMemcpyAsync(depth, d_dp, sizeof(float) * nL, cudaMemcpyDeviceToHost, m->stream));
    }
    ORBGPU_CUDA_TRY(cudaMemcpyAsync(m->h_pinned, status, sizeof(int), cudaMemcpyDeviceToHost, m->stream));
    ORBGPU_CUDA_TRY(cudaStreamSynchronize(m->stream));
    if (m->h_pinned[0]) {
        orbgpu_set_last_error("stereo patch outside its level", __FILE__, __LINE__);
        return ORBGPU_ERR_BAD_ARG;
    }
    return ORBGPU_OK;
}

extern "C" int orbgpu_descriptor_distance(const uint8_t* a, const uint8_t* b, int n, int* out, void* stream) {
    if (n < 0 || (n > 0 && (!a || !b || !out))) return ORBGPU_ERR_BAD_ARG;
    if (n == 0) return ORBGPU_OK;
    k_descriptor_distance<<<(n + 255) / 256, 256, 0, (cudaStream_t)stream>>>(a, b, n, out);
    ORBGPU_CUDA_TRY(cudaGetLastError());
    return ORBGPU_OK;
}

// ---------------------------------------------------------------- internal access for the kNN file
cudaStream_t orbgpu_matcher_stream_internal(orbgpu_matcher* m) { return m->stream; }
