// orb_oracle.cpp -- ORACLE / TEST INFRASTRUCTURE ONLY.
//
// CPU restatement of ORB-SLAM2's feature front-end (see orb_oracle.h).  The
// code is this repository's own; each function names the reference lines it
// restates.  OpenCV primitives come from cvshim/cvshim_prims.h.
//
// DistributeOctTree is restated with explicit node creation numbers instead of
// list node addresses: the reference's list only ever grows at the front
// after the initial nodes are appended, so list order is "non-initial nodes by
// creation number descending, then initial nodes ascending", and the
// (size, node*) sort at src/ORBextractor.cc:926 breaks size ties by creation
// order once allocation order is made monotonic.
#include "orb_oracle.h"

#include <algorithm>
#include <array>
#include <fstream>
#include <map>
#include <sstream>
#include <string>
#include <climits>
#include <cmath>
#include <cstring>
#include <vector>

#include "cvshim/cvshim_prims.h"
#include "orb_pattern_table.h"

namespace {

const int kEdgeThreshold = 19;
const int kHalfPatch = 15;
const int kPatchSize = 31;
const int kGridCols = 64;
const int kGridRows = 48;
const int kThHigh = 100;
const int kThLow = 50;
const int kHistoLength = 30;

struct Tables {
    int nlevels;
    std::vector<float> scale, inv_scale, sigma2, inv_sigma2;
    std::vector<int> nfeat;
    int umax[kHalfPatch + 1];
};

// ORBextractor::ORBextractor, src/ORBextractor.cc:469-571.
Tables make_tables(const orc_params* p) {
    Tables t;
    t.nlevels = p->nlevels;
    const double sf = (double)p->scale_factor;  // scaleFactor is a double member
    t.scale.assign(p->nlevels, 1.0f);
    t.sigma2.assign(p->nlevels, 1.0f);
    for (int i = 1; i < p->nlevels; i++) {
        t.scale[i] = (float)(t.scale[i - 1] * sf);
        t.sigma2[i] = t.scale[i] * t.scale[i];
    }
    t.inv_scale.resize(p->nlevels);
    t.inv_sigma2.resize(p->nlevels);
    for (int i = 0; i < p->nlevels; i++) {
        t.inv_scale[i] = 1.0f / t.scale[i];
        t.inv_sigma2[i] = 1.0f / t.sigma2[i];
    }
    t.nfeat.assign(p->nlevels, 0);
    const float factor = (float)(1.0f / sf);
    float per_scale = p->nfeatures * (1 - factor) / (1 - (float)std::pow((double)factor, (double)p->nlevels));
    int sum = 0;
    for (int l = 0; l < p->nlevels - 1; l++) {
        t.nfeat[l] = shim_cvround_f(per_scale);
        sum += t.nfeat[l];
        per_scale *= factor;
    }
    t.nfeat[p->nlevels - 1] = std::max(p->nfeatures - sum, 0);
    const int vmax = (int)std::floor(kHalfPatch * std::sqrt(2.f) / 2 + 1);
    const int vmin = (int)std::ceil(kHalfPatch * std::sqrt(2.f) / 2);
    const double hp2 = kHalfPatch * kHalfPatch;
    for (int v = 0; v <= vmax; ++v) t.umax[v] = shim_cvround_d(std::sqrt(hp2 - v * v));
    for (int v = kHalfPatch, v0 = 0; v >= vmin; --v) {
        while (t.umax[v0] == t.umax[v0 + 1]) ++v0;
        t.umax[v] = v0;
        ++v0;
    }
    return t;
}

struct Level {
    int w, h;
    std::vector<uint8_t> px;
    const uint8_t* at(int x, int y) const { return &px[(size_t)y * w + x]; }
};

// ComputePyramid, src/ORBextractor.cc:1655-1724 (the padded border is never
// read on the path, so only the level interiors are kept).
std::vector<Level> build_pyramid(const uint8_t* img, int w, int h, size_t step, const Tables& t) {
    std::vector<Level> pyr(t.nlevels);
    for (int l = 0; l < t.nlevels; l++) {
        const float s = t.inv_scale[l];
        Level& L = pyr[l];
        L.w = shim_cvround_f((float)w * s);
        L.h = shim_cvround_f((float)h * s);
        L.px.resize((size_t)L.w * L.h);
        if (l == 0) {
            for (int y = 0; y < h; y++) std::memcpy(&L.px[(size_t)y * w], img + (size_t)y * step, w);
        } else {
            const Level& P = pyr[l - 1];
            shim_resize_linear_u8(P.px.data(), P.w, P.w, P.h, L.px.data(), L.w, L.w, L.h);
        }
    }
    return pyr;
}

// The per-cell FAST loop of ComputeKeyPointsOctTree, src/ORBextractor.cc:1069-1142.
std::vector<orc_kp> fast_level(const Level& L, int ini_th, int min_th) {
    std::vector<orc_kp> out;
    const int minBorderX = kEdgeThreshold - 3, minBorderY = minBorderX;
    const int maxBorderX = L.w - kEdgeThreshold + 3, maxBorderY = L.h - kEdgeThreshold + 3;
    const float W = 30;
    const float width = (float)(maxBorderX - minBorderX), height = (float)(maxBorderY - minBorderY);
    const int nCols = (int)(width / W), nRows = (int)(height / W);
    if (nCols <= 0 || nRows <= 0) return out;
    const int wCell = (int)std::ceil(width / nCols), hCell = (int)std::ceil(height / nRows);
    std::vector<shim_corner> buf;
    for (int i = 0; i < nRows; i++) {
        const float iniY = (float)(minBorderY + i * hCell);
        float maxY = iniY + hCell + 6;
        if (iniY >= maxBorderY - 3) continue;
        if (maxY > maxBorderY) maxY = (float)maxBorderY;
        for (int j = 0; j < nCols; j++) {
            const float iniX = (float)(minBorderX + j * wCell);
            float maxX = iniX + wCell + 6;
            if (iniX >= maxBorderX - 6) continue;
            if (maxX > maxBorderX) maxX = (float)maxBorderX;
            const int y0 = (int)iniY, y1 = (int)maxY, x0 = (int)iniX, x1 = (int)maxX;
            const int rw = x1 - x0, rh = y1 - y0;
            buf.resize((size_t)rw * rh / 4 + 16);
            const uint8_t* roi = L.at(x0, y0);
            int n = shim_fast9_u8(roi, L.w, rw, rh, ini_th, buf.data(), (int)buf.size());
            if (n == 0) n = shim_fast9_u8(roi, L.w, rw, rh, min_th, buf.data(), (int)buf.size());
            for (int k = 0; k < n; k++) {
                orc_kp kp;
                kp.x = (float)buf[k].x + (float)(j * wCell);
                kp.y = (float)buf[k].y + (float)(i * hCell);
                kp.size = 7.f;
                kp.angle = -1.f;
                kp.response = (float)buf[k].score;
                kp.octave = 0;
                kp.class_id = -1;
                out.push_back(kp);
            }
        }
    }
    return out;
}

struct Node {
    int x0, x1, y0, y1;     // UL.x, UR.x, UL.y, BR.y
    std::vector<int> keys;  // indices into the candidate list, in list order
    bool no_more = false;
    bool alive = true;
    bool root = false;
    long id = 0;
};

// ExtractorNode::DivideNode, src/ORBextractor.cc:602-674.
void divide(const Node& p, const std::vector<orc_kp>& c, Node ch[4]) {
    const int halfX = (int)std::ceil(static_cast<float>(p.x1 - p.x0) / 2);
    const int halfY = (int)std::ceil(static_cast<float>(p.y1 - p.y0) / 2);
    const int xm = p.x0 + halfX, ym = p.y0 + halfY;
    ch[0].x0 = p.x0; ch[0].x1 = xm;   ch[0].y0 = p.y0; ch[0].y1 = ym;
    ch[1].x0 = xm;   ch[1].x1 = p.x1; ch[1].y0 = p.y0; ch[1].y1 = ym;
    ch[2].x0 = p.x0; ch[2].x1 = xm;   ch[2].y0 = ym;   ch[2].y1 = p.y1;
    ch[3].x0 = xm;   ch[3].x1 = p.x1; ch[3].y0 = ym;   ch[3].y1 = p.y1;
    for (int k : p.keys) {
        const orc_kp& kp = c[k];
        int q;
        if (kp.x < (float)xm) q = kp.y < (float)ym ? 0 : 2;
        else q = kp.y < (float)ym ? 1 : 3;
        ch[q].keys.push_back(k);
    }
    for (int q = 0; q < 4; q++)
        if (ch[q].keys.size() == 1) ch[q].no_more = true;
}

// DistributeOctTree, src/ORBextractor.cc:688-1033.
std::vector<orc_kp> distribute(const std::vector<orc_kp>& cand, int minX, int maxX, int minY, int maxY, int N) {
    const int nIni = (int)std::round(static_cast<float>(maxX - minX) / (maxY - minY));
    const float hX = static_cast<float>(maxX - minX) / nIni;
    std::vector<Node> nodes;
    long next_id = 0;
    for (int i = 0; i < nIni; i++) {
        Node n;
        n.x0 = (int)(hX * static_cast<float>(i));
        n.x1 = (int)(hX * static_cast<float>(i + 1));
        n.y0 = 0;
        n.y1 = maxY - minY;
        n.root = true;
        n.id = next_id++;
        nodes.push_back(n);
    }
    for (size_t i = 0; i < cand.size(); i++) nodes[(size_t)(cand[i].x / hX)].keys.push_back((int)i);
    for (Node& n : nodes) {
        if (n.keys.size() == 1) n.no_more = true;
        else if (n.keys.empty()) n.alive = false;
    }
    int alive = 0;
    for (const Node& n : nodes) alive += n.alive;

    auto list_order = [&]() {
        std::vector<int> ord;
        for (int i = 0; i < (int)nodes.size(); i++)
            if (nodes[i].alive) ord.push_back(i);
        std::sort(ord.begin(), ord.end(), [&](int a, int b) {
            const Node &A = nodes[a], &B = nodes[b];
            if (A.root != B.root) return !A.root;
            return A.root ? A.id < B.id : A.id > B.id;
        });
        return ord;
    };
    // Splits node idx, creating its non-empty children in n1..n4 order;
    // returns the indices of the children holding more than one key.
    auto split = [&](int idx, std::vector<int>& big) {
        Node ch[4];
        divide(nodes[idx], cand, ch);
        nodes[idx].alive = false;
        alive--;
        for (int q = 0; q < 4; q++) {
            if (ch[q].keys.empty()) continue;
            ch[q].id = next_id++;
            nodes.push_back(ch[q]);
            alive++;
            if (nodes.back().keys.size() > 1) big.push_back((int)nodes.size() - 1);
        }
    };

    bool finish = false;
    std::vector<int> expand;
    while (!finish) {
        int prev = alive;
        std::vector<int> ord = list_order();
        expand.clear();
        for (int idx : ord) {
            if (nodes[idx].no_more) continue;
            split(idx, expand);
        }
        const int nToExpand = (int)expand.size();
        if (alive >= N || alive == prev) {
            finish = true;
        } else if (alive + nToExpand * 3 > N) {
            while (!finish) {
                prev = alive;
                std::vector<int> vprev = expand;
                expand.clear();
                std::sort(vprev.begin(), vprev.end(), [&](int a, int b) {
                    if (nodes[a].keys.size() != nodes[b].keys.size()) return nodes[a].keys.size() < nodes[b].keys.size();
                    return nodes[a].id < nodes[b].id;
                });
                for (int j = (int)vprev.size() - 1; j >= 0; j--) {
                    split(vprev[j], expand);
                    if (alive >= N) break;
                }
                if (alive >= N || alive == prev) finish = true;
            }
        }
    }
    std::vector<orc_kp> res;
    for (int idx : list_order()) {
        const Node& n = nodes[idx];
        int best = n.keys[0];
        float maxr = cand[best].response;
        for (size_t k = 1; k < n.keys.size(); k++)
            if (cand[n.keys[k]].response > maxr) {
                best = n.keys[k];
                maxr = cand[best].response;
            }
        res.push_back(cand[best]);
    }
    return res;
}

// IC_Angle, src/ORBextractor.cc:94-141.
float ic_angle(const Level& L, float px, float py, const int* umax) {
    int m_01 = 0, m_10 = 0;
    const uint8_t* center = L.at(shim_cvround_f(px), shim_cvround_f(py));
    for (int u = -kHalfPatch; u <= kHalfPatch; ++u) m_10 += u * center[u];
    const int step = L.w;
    for (int v = 1; v <= kHalfPatch; ++v) {
        int v_sum = 0;
        const int d = umax[v];
        for (int u = -d; u <= d; ++u) {
            const int vp = center[u + v * step], vm = center[u - v * step];
            v_sum += vp - vm;
            m_10 += u * (vp + vm);
        }
        m_01 += v * v_sum;
    }
    return shim_fast_atan2((float)m_01, (float)m_10);
}

// computeOrbDescriptor, src/ORBextractor.cc:153-204 (on the blurred level).
void orb_descriptor(const orc_kp& kp, const uint8_t* blurred, int w, uint8_t* desc) {
    const float factorPI = (float)(3.1415926535897932384626433832795 / 180.f);
    const float angle = (float)kp.angle * factorPI;
    const float a = (float)cosf(angle), b = (float)sinf(angle);
    const uint8_t* center = blurred + (size_t)shim_cvround_f(kp.y) * w + shim_cvround_f(kp.x);
    const int step = w;
    for (int i = 0; i < 32; ++i) {
        int val = 0;
        for (int k = 0; k < 8; k++) {
            const signed char* pp = &kOracleBriefPattern[(i * 16 + 2 * k) * 2];
            int t[2];
            for (int e = 0; e < 2; e++) {
                const float x = (float)pp[2 * e], y = (float)pp[2 * e + 1];
                t[e] = center[shim_cvround_f(x * b + y * a) * step + shim_cvround_f(x * a - y * b)];
            }
            val |= (t[0] < t[1]) << k;
        }
        desc[i] = (uint8_t)val;
    }
}

struct Grid {
    float minX, maxX, minY, maxY, invW, invH;
    std::vector<int> cells[kGridCols][kGridRows];
};

// ComputeImageBounds (no distortion) + grid constants + AssignFeaturesToGrid,
// src/Frame.cc:783-819, :372-388, :399-423, PosInGrid :682-698.
void build_grid(Grid& g, const orc_kp* kps, int n, int w, int h) {
    g.minX = 0.0f;
    g.maxX = (float)w;
    g.minY = 0.0f;
    g.maxY = (float)h;
    g.invW = static_cast<float>(kGridCols) / static_cast<float>(g.maxX - g.minX);
    g.invH = static_cast<float>(kGridRows) / static_cast<float>(g.maxY - g.minY);
    for (int i = 0; i < n; i++) {
        const int px = (int)std::round((kps[i].x - g.minX) * g.invW);
        const int py = (int)std::round((kps[i].y - g.minY) * g.invH);
        if (px < 0 || px >= kGridCols || py < 0 || py >= kGridRows) continue;
        g.cells[px][py].push_back(i);
    }
}

// Frame::GetFeaturesInArea, src/Frame.cc:590-670.
std::vector<int> features_in_area(const Grid& g, const orc_kp* kps, float x, float y, float r, int minLevel,
                                  int maxLevel) {
    std::vector<int> v;
    const int nMinCellX = std::max(0, (int)std::floor((x - g.minX - r) * g.invW));
    if (nMinCellX >= kGridCols) return v;
    const int nMaxCellX = std::min(kGridCols - 1, (int)std::ceil((x - g.minX + r) * g.invW));
    if (nMaxCellX < 0) return v;
    const int nMinCellY = std::max(0, (int)std::floor((y - g.minY - r) * g.invH));
    if (nMinCellY >= kGridRows) return v;
    const int nMaxCellY = std::min(kGridRows - 1, (int)std::ceil((y - g.minY + r) * g.invH));
    if (nMaxCellY < 0) return v;
    const bool check = (minLevel > 0) || (maxLevel >= 0);
    for (int ix = nMinCellX; ix <= nMaxCellX; ix++)
        for (int iy = nMinCellY; iy <= nMaxCellY; iy++)
            for (int idx : g.cells[ix][iy]) {
                const orc_kp& kp = kps[idx];
                if (check) {
                    if (kp.octave < minLevel) continue;
                    if (maxLevel >= 0 && kp.octave > maxLevel) continue;
                }
                const float dx = kp.x - x, dy = kp.y - y;
                if (dx * dx + dy * dy < r * r) v.push_back(idx);
            }
    return v;
}

// ORBmatcher::DescriptorDistance, src/ORBmatcher.cc:2083-2103.
int hamming(const uint8_t* a, const uint8_t* b) {
    int d = 0;
    for (int i = 0; i < 8; i++) {
        uint32_t x, y;
        std::memcpy(&x, a + 4 * i, 4);
        std::memcpy(&y, b + 4 * i, 4);
        d += __builtin_popcount(x ^ y);
    }
    return d;
}

// ORBmatcher::ComputeThreeMaxima, src/ORBmatcher.cc:2035-2077.
void three_maxima(const std::vector<int>* histo, int L, int& ind1, int& ind2, int& ind3) {
    int max1 = 0, max2 = 0, max3 = 0;
    for (int i = 0; i < L; i++) {
        const int s = (int)histo[i].size();
        if (s > max1) {
            max3 = max2; max2 = max1; max1 = s;
            ind3 = ind2; ind2 = ind1; ind1 = i;
        } else if (s > max2) {
            max3 = max2; max2 = s;
            ind3 = ind2; ind2 = i;
        } else if (s > max3) {
            max3 = s;
            ind3 = i;
        }
    }
    if (max2 < 0.1f * (float)max1) {
        ind2 = -1;
        ind3 = -1;
    } else if (max3 < 0.1f * (float)max1) {
        ind3 = -1;
    }
}

}  // namespace

extern "C" {

// ORBextractor::operator(), src/ORBextractor.cc:1533-1649.
int orc_extract(const uint8_t* img, int w, int h, size_t step, const orc_params* p, orc_kp* kps, uint8_t* desc,
                int cap, int* n_out, uint8_t* pyr_out, size_t pyr_cap) {
    *n_out = 0;
    if (img == nullptr || w <= 0 || h <= 0) return 0;
    const Tables t = make_tables(p);
    const std::vector<Level> pyr = build_pyramid(img, w, h, step, t);
    std::vector<std::vector<orc_kp> > all(t.nlevels);
    for (int l = 0; l < t.nlevels; l++) {
        const Level& L = pyr[l];
        std::vector<orc_kp> cand = fast_level(L, p->ini_th_fast, p->min_th_fast);
        const int minBorderX = kEdgeThreshold - 3, minBorderY = minBorderX;
        const int maxBorderX = L.w - kEdgeThreshold + 3, maxBorderY = L.h - kEdgeThreshold + 3;
        std::vector<orc_kp> keys = distribute(cand, minBorderX, maxBorderX, minBorderY, maxBorderY, t.nfeat[l]);
        const int scaledPatchSize = (int)(kPatchSize * t.scale[l]);
        for (orc_kp& k : keys) {
            k.x += minBorderX;
            k.y += minBorderY;
            k.octave = l;
            k.size = (float)scaledPatchSize;
        }
        for (orc_kp& k : keys) k.angle = ic_angle(L, k.x, k.y, t.umax);
        all[l] = keys;
    }
    int total = 0;
    for (auto& v : all) total += (int)v.size();
    *n_out = total;
    if (total > cap) return -1;
    int off = 0;
    for (int l = 0; l < t.nlevels; l++) {
        std::vector<orc_kp>& keys = all[l];
        if (keys.empty()) continue;
        const Level& L = pyr[l];
        std::vector<uint8_t> blurred(L.px.size());
        shim_gauss7_u8(L.px.data(), L.w, L.w, L.h, blurred.data(), L.w);
        for (size_t i = 0; i < keys.size(); i++) orb_descriptor(keys[i], blurred.data(), L.w, desc + (size_t)(off + i) * 32);
        if (l != 0) {
            const float s = t.scale[l];
            for (orc_kp& k : keys) {
                k.x *= s;
                k.y *= s;
            }
        }
        for (size_t i = 0; i < keys.size(); i++) kps[off + i] = keys[i];
        off += (int)keys.size();
    }
    if (pyr_out) {
        size_t o = 0;
        for (const Level& L : pyr) {
            if (o + L.px.size() > pyr_cap) return -2;
            std::memcpy(pyr_out + o, L.px.data(), L.px.size());
            o += L.px.size();
        }
    }
    return 0;
}

int orc_extractor_tables(const orc_params* p, float* scale, float* inv_scale, float* sigma2, float* inv_sigma2,
                         int* features_per_level, int* umax16) {
    const Tables t = make_tables(p);
    for (int l = 0; l < p->nlevels; l++) {
        scale[l] = t.scale[l];
        inv_scale[l] = t.inv_scale[l];
        sigma2[l] = t.sigma2[l];
        inv_sigma2[l] = t.inv_sigma2[l];
        features_per_level[l] = t.nfeat[l];
    }
    for (int v = 0; v < 16; v++) umax16[v] = t.umax[v];
    return 0;
}

int orc_descriptor_distance(const uint8_t* a, const uint8_t* b) { return hamming(a, b); }

int orc_features_in_area(const orc_params* p, const orc_kp* kps, int n, int w, int h, float x, float y, float r,
                         int minLevel, int maxLevel, int* out, int cap) {
    (void)p;
    Grid* g = new Grid();
    build_grid(*g, kps, n, w, h);
    std::vector<int> v = features_in_area(*g, kps, x, y, r, minLevel, maxLevel);
    delete g;
    for (int i = 0; i < (int)v.size() && i < cap; i++) out[i] = v[i];
    return (int)v.size();
}

// ORBmatcher::SearchForInitialization, src/ORBmatcher.cc:573-717.
int orc_search_for_initialization(const orc_params* p, const orc_kp* kps1, const uint8_t* desc1, int n1,
                                  const orc_kp* kps2, const uint8_t* desc2, int n2, int w, int h,
                                  float* prev_matched_xy, int window, float nnratio, int check_ori, int* matches12) {
    (void)p;
    Grid* g2 = new Grid();
    build_grid(*g2, kps2, n2, w, h);
    int nmatches = 0;
    for (int i = 0; i < n1; i++) matches12[i] = -1;
    std::vector<int> rotHist[kHistoLength];
    const float factor = kHistoLength / 360.0f;
    std::vector<int> matchedDistance(n2, INT_MAX), matches21(n2, -1);
    for (int i1 = 0; i1 < n1; i1++) {
        const orc_kp kp1 = kps1[i1];
        const int level1 = kp1.octave;
        if (level1 > 0) continue;
        std::vector<int> idx2 = features_in_area(*g2, kps2, prev_matched_xy[2 * i1], prev_matched_xy[2 * i1 + 1],
                                                 (float)window, level1, level1);
        if (idx2.empty()) continue;
        int bestDist = INT_MAX, bestDist2 = INT_MAX, bestIdx2 = -1;
        for (int i2 : idx2) {
            const int dist = hamming(desc1 + (size_t)i1 * 32, desc2 + (size_t)i2 * 32);
            if (matchedDistance[i2] <= dist) continue;
            if (dist < bestDist) {
                bestDist2 = bestDist;
                bestDist = dist;
                bestIdx2 = i2;
            } else if (dist < bestDist2) {
                bestDist2 = dist;
            }
        }
        if (bestDist <= kThLow && bestDist < (float)bestDist2 * nnratio) {
            if (matches21[bestIdx2] >= 0) {
                matches12[matches21[bestIdx2]] = -1;
                nmatches--;
            }
            matches12[i1] = bestIdx2;
            matches21[bestIdx2] = i1;
            matchedDistance[bestIdx2] = bestDist;
            nmatches++;
            if (check_ori) {
                float rot = kps1[i1].angle - kps2[bestIdx2].angle;
                if (rot < 0.0) rot += 360.0f;
                int bin = (int)std::round(rot * factor);
                if (bin == kHistoLength) bin = 0;
                rotHist[bin].push_back(i1);
            }
        }
    }
    if (check_ori) {
        int ind1 = -1, ind2 = -1, ind3 = -1;
        three_maxima(rotHist, kHistoLength, ind1, ind2, ind3);
        for (int i = 0; i < kHistoLength; i++) {
            if (i == ind1 || i == ind2 || i == ind3) continue;
            for (int idx1 : rotHist[i])
                if (matches12[idx1] >= 0) {
                    matches12[idx1] = -1;
                    nmatches--;
                }
        }
    }
    for (int i1 = 0; i1 < n1; i1++)
        if (matches12[i1] >= 0) {
            prev_matched_xy[2 * i1] = kps2[matches12[i1]].x;
            prev_matched_xy[2 * i1 + 1] = kps2[matches12[i1]].y;
        }
    delete g2;
    return nmatches;
}

// ORBmatcher::SearchByProjection(Frame&, const vector<MapPoint*>&, th),
// src/ORBmatcher.cc:72-183, with RadiusByViewingCos :186-193.
int orc_search_by_projection(const orc_params* p, const orc_kp* kps, const uint8_t* desc, const float* uright, int n,
                             int w, int h, const orc_mappoint* mps, const uint8_t* mp_desc, int m, float th,
                             float nnratio, const uint8_t* claimed, int* match_out) {
    const Tables t = make_tables(p);
    Grid* g = new Grid();
    build_grid(*g, kps, n, w, h);
    for (int i = 0; i < n; i++) match_out[i] = (claimed && claimed[i]) ? -2 : -1;
    int nmatches = 0;
    const bool bFactor = th != 1.0;
    for (int imp = 0; imp < m; imp++) {
        const orc_mappoint& mp = mps[imp];
        if (!mp.track_in_view || mp.bad) continue;
        const int level = mp.track_scale_level;
        float r = mp.view_cos > 0.998 ? 2.5f : 4.0f;
        if (bFactor) r *= th;
        const float radius = r * t.scale[level];
        std::vector<int> idx = features_in_area(*g, kps, mp.proj_x, mp.proj_y, radius, level - 1, level);
        if (idx.empty()) continue;
        int bestDist = 256, bestLevel = -1, bestDist2 = 256, bestLevel2 = -1, bestIdx = -1;
        for (int i : idx) {
            if (match_out[i] != -1) continue;
            if (uright && uright[i] > 0) {
                const float er = std::fabs(mp.proj_xr - uright[i]);
                if (er > r * t.scale[level]) continue;
            }
            const int dist = hamming(mp_desc + (size_t)imp * 32, desc + (size_t)i * 32);
            if (dist < bestDist) {
                bestDist2 = bestDist;
                bestDist = dist;
                bestLevel2 = bestLevel;
                bestLevel = kps[i].octave;
                bestIdx = i;
            } else if (dist < bestDist2) {
                bestLevel2 = kps[i].octave;
                bestDist2 = dist;
            }
        }
        if (bestDist <= kThHigh) {
            if (bestLevel == bestLevel2 && bestDist > nnratio * bestDist2) continue;
            match_out[bestIdx] = imp;
            nmatches++;
        }
    }
    delete g;
    return nmatches;
}

// KeyFrame::GetFeaturesInArea, src/KeyFrame.cc:785-830: the same cells as
// the frame's, but a square window (|dx| < r and |dy| < r) where this tree's
// Frame::GetFeaturesInArea keeps a disc.
static std::vector<int> kf_features_in_area(const Grid& g, const orc_kp* kps, float x, float y, float r) {
    std::vector<int> v;
    const int x0 = std::max(0, (int)std::floor((x - g.minX - r) * g.invW));
    if (x0 >= kGridCols) return v;
    const int x1 = std::min(kGridCols - 1, (int)std::ceil((x - g.minX + r) * g.invW));
    if (x1 < 0) return v;
    const int y0 = std::max(0, (int)std::floor((y - g.minY - r) * g.invH));
    if (y0 >= kGridRows) return v;
    const int y1 = std::min(kGridRows - 1, (int)std::ceil((y - g.minY + r) * g.invH));
    if (y1 < 0) return v;
    for (int ix = x0; ix <= x1; ix++)
        for (int iy = y0; iy <= y1; iy++)
            for (int idx : g.cells[ix][iy])
                if (std::fabs(kps[idx].x - x) < r && std::fabs(kps[idx].y - y) < r) v.push_back(idx);
    return v;
}

// cv::Mat products of the reference's pose algebra: the 3 x 3 float product
// accumulates in double and is stored as float (gemm), an added vector is a
// float addition.
static float mat_row_dot(const float* row, int stride, const float* x) {
    double s = 0.0;
    for (int k = 0; k < 3; k++) s += (double)row[k * stride] * (double)x[k];
    return (float)s;
}

// ORBmatcher::SearchByProjection(Frame& CurrentFrame, const Frame& LastFrame,
// th, bMono), src/ORBmatcher.cc:1710-1879.
int orc_search_by_projection_frame(const orc_params* p, const orc_kp* kps, const uint8_t* desc, const float* uright,
                                   int n, int w, int h, const orc_kp* last_kps, int n_last,
                                   const orc_frame_mappoint* last_mps, const uint8_t* last_mp_desc,
                                   const orc_frame_motion* mo, float th, int mono, int check_ori,
                                   const uint8_t* claimed, int* match_out) {
    const Tables t = make_tables(p);
    Grid* g = new Grid();
    build_grid(*g, kps, n, w, h);
    // mvpMapPoints of the current frame: -1 none, -2 pre-claimed (observed), >= 0 LastFrame index
    std::vector<int> owner(n);
    for (int i = 0; i < n; i++) owner[i] = (claimed && claimed[i]) ? -2 : -1;
    std::vector<char> touched(n, 0);
    std::vector<int> rotHist[kHistoLength];
    const float factor = kHistoLength / 360.0f;
    // twc = -Rcw' tcw, tlc = Rlw twc + tlw (src/ORBmatcher.cc:1724-1737)
    const float* T = mo->Tcw;
    const float tcw[3] = {T[3], T[7], T[11]};
    float twc[3];
    for (int r = 0; r < 3; r++) {
        const float col[3] = {-T[r], -T[4 + r], -T[8 + r]};  // row r of -Rcw'
        twc[r] = mat_row_dot(col, 1, tcw);
    }
    const float* L = mo->Tlw;
    const float tlcz = mat_row_dot(L + 8, 1, twc) + L[11];
    const bool bForward = tlcz > mo->b && !mono;
    const bool bBackward = -tlcz > mo->b && !mono;
    int nmatches = 0;
    for (int i = 0; i < n_last; i++) {
        const orc_frame_mappoint& mp = last_mps[i];
        if (!(mp.flags & ORC_MP_PRESENT) || (mp.flags & ORC_MP_OUTLIER)) continue;
        const float X[3] = {mp.x, mp.y, mp.z};
        float c[3];
        for (int r = 0; r < 3; r++) c[r] = mat_row_dot(T + 4 * r, 1, X) + T[4 * r + 3];
        const float xc = c[0], yc = c[1];
        const float invzc = 1.0 / c[2];
        if (invzc < 0) continue;
        const float u = mo->fx * xc * invzc + mo->cx;
        const float v = mo->fy * yc * invzc + mo->cy;
        // a non-finite projection finds no cell in the reference (x86 float->int of NaN)
        if (!std::isfinite(u) || !std::isfinite(v)) continue;
        if (u < g->minX || u > g->maxX) continue;
        if (v < g->minY || v > g->maxY) continue;
        const int nLastOctave = last_kps[i].octave;
        const float radius = th * t.scale[nLastOctave];
        std::vector<int> idx2;
        if (bForward) idx2 = features_in_area(*g, kps, u, v, radius, nLastOctave, -1);
        else if (bBackward) idx2 = features_in_area(*g, kps, u, v, radius, 0, nLastOctave);
        else idx2 = features_in_area(*g, kps, u, v, radius, nLastOctave - 1, nLastOctave + 1);
        if (idx2.empty()) continue;
        int bestDist = 256, bestIdx2 = -1;
        for (int i2 : idx2) {
            // an owner with observations blocks (src/ORBmatcher.cc:1800-1802)
            if (owner[i2] == -2 || (owner[i2] >= 0 && (last_mps[owner[i2]].flags & ORC_MP_OBSERVED))) continue;
            if (uright && uright[i2] > 0) {
                const float ur = u - mo->bf * invzc;
                const float er = std::fabs(ur - uright[i2]);
                if (er > radius) continue;
            }
            const int dist = hamming(last_mp_desc + (size_t)i * 32, desc + (size_t)i2 * 32);
            if (dist < bestDist) {
                bestDist = dist;
                bestIdx2 = i2;
            }
        }
        if (bestDist <= kThHigh) {
            owner[bestIdx2] = i;
            touched[bestIdx2] = 1;
            nmatches++;
            if (check_ori) {
                float rot = last_kps[i].angle - kps[bestIdx2].angle;
                if (rot < 0.0) rot += 360.0f;
                int bin = (int)std::round(rot * factor);
                if (bin == kHistoLength) bin = 0;
                rotHist[bin].push_back(bestIdx2);
            }
        }
    }
    std::vector<char> nulled(n, 0);
    if (check_ori) {
        int ind1 = -1, ind2 = -1, ind3 = -1;
        three_maxima(rotHist, kHistoLength, ind1, ind2, ind3);
        for (int b = 0; b < kHistoLength; b++) {
            if (b == ind1 || b == ind2 || b == ind3) continue;
            for (int i2 : rotHist[b]) {
                nulled[i2] = 1;
                nmatches--;
            }
        }
    }
    for (int i = 0; i < n; i++) match_out[i] = nulled[i] ? -4 : owner[i];
    delete g;
    return nmatches;
}

// ORBmatcher::SearchByProjection(Frame& CurrentFrame, KeyFrame* pKF,
// sAlreadyFound, th, ORBdist), src/ORBmatcher.cc:1891-2010.  T: rows 0-2 of
// CurrentFrame.mTcw; cam = fx, fy, cx, cy.  mp_state: 0 no map point, 1
// usable, 2 bad, 3 in sAlreadyFound.  match_out as the frame-to-frame search
// (-4 assigned then reset by the rotation check).
int orc_search_by_projection_kf(const orc_params* p, const orc_kp* kps, const uint8_t* desc, int n, int w, int h,
                                const float* T, const float* cam, const orc_kp* kf_kps, int m,
                                const orc_mp_geometry* mps, const uint8_t* mp_desc, const uint8_t* mp_state, float th,
                                int orbdist, int check_ori, const uint8_t* claimed, int* match_out) {
    const Tables t = make_tables(p);
    Grid* g = new Grid();
    build_grid(*g, kps, n, w, h);
    std::vector<int> owner(n);
    for (int i = 0; i < n; i++) owner[i] = (claimed && claimed[i]) ? -2 : -1;
    std::vector<int> rotHist[kHistoLength];
    const float factor = kHistoLength / 360.0f;
    // Ow = -Rcw' tcw
    const float tcw[3] = {T[3], T[7], T[11]};
    float Ow[3];
    for (int r = 0; r < 3; r++) {
        const float col[3] = {-T[r], -T[4 + r], -T[8 + r]};
        Ow[r] = mat_row_dot(col, 1, tcw);
    }
    const float log_scale = std::log(p->scale_factor);
    int nmatches = 0;
    for (int i = 0; i < m; i++) {
        if (mp_state[i] != 1) continue;
        const orc_mp_geometry& mp = mps[i];
        const float X[3] = {mp.x, mp.y, mp.z};
        float c[3];
        for (int r = 0; r < 3; r++) c[r] = mat_row_dot(T + 4 * r, 1, X) + T[4 * r + 3];
        const float invzc = 1.0 / c[2];
        const float u = cam[0] * c[0] * invzc + cam[2];
        const float v = cam[1] * c[1] * invzc + cam[3];
        // a non-finite projection finds no cell in the reference
        if (!std::isfinite(u) || !std::isfinite(v)) continue;
        if (u < g->minX || u > g->maxX) continue;
        if (v < g->minY || v > g->maxY) continue;
        const float PO[3] = {X[0] - Ow[0], X[1] - Ow[1], X[2] - Ow[2]};
        double ss = 0;
        for (int k = 0; k < 3; k++) ss += (double)PO[k] * (double)PO[k];
        const float dist3D = (float)std::sqrt(ss);
        if (dist3D < 0.8f * mp.min_distance || dist3D > 1.2f * mp.max_distance) continue;
        const float ratio = mp.max_distance / dist3D;
        int level = (int)std::ceil(std::log(ratio) / log_scale);
        if (level < 0) level = 0;
        else if (level >= p->nlevels) level = p->nlevels - 1;
        const float radius = th * t.scale[level];
        const std::vector<int> idx2 = features_in_area(*g, kps, u, v, radius, level - 1, level + 1);
        if (idx2.empty()) continue;
        int bestDist = 256, bestIdx2 = -1;
        for (int i2 : idx2) {
            if (owner[i2] != -1) continue;  // CurrentFrame.mvpMapPoints[i2] set
            const int dist = hamming(mp_desc + (size_t)i * 32, desc + (size_t)i2 * 32);
            if (dist < bestDist) {
                bestDist = dist;
                bestIdx2 = i2;
            }
        }
        if (bestDist <= orbdist) {
            owner[bestIdx2] = i;
            nmatches++;
            if (check_ori) {
                float rot = kf_kps[i].angle - kps[bestIdx2].angle;
                if (rot < 0.0) rot += 360.0f;
                int bin = (int)std::round(rot * factor);
                if (bin == kHistoLength) bin = 0;
                rotHist[bin].push_back(bestIdx2);
            }
        }
    }
    std::vector<char> nulled(n, 0);
    if (check_ori) {
        int ind1 = -1, ind2 = -1, ind3 = -1;
        three_maxima(rotHist, kHistoLength, ind1, ind2, ind3);
        for (int b = 0; b < kHistoLength; b++) {
            if (b == ind1 || b == ind2 || b == ind3) continue;
            for (int i2 : rotHist[b]) {
                nulled[i2] = 1;
                nmatches--;
            }
        }
    }
    for (int i = 0; i < n; i++) match_out[i] = nulled[i] ? -4 : owner[i];
    delete g;
    return nmatches;
}

// ORBmatcher::SearchForTriangulation(pKF1, pKF2, F12, vMatchedPairs,
// bOnlyStereo), src/ORBmatcher.cc:884-1040, with CheckDistEpipolarLine
// (:205-232).  Features without a map point only (mp != 0 is a map point,
// bad or not); in a common node every pKF1 feature takes, among the node's
// unmatched pKF2 features at distance <= TH_LOW passing the epipole distance
// (both monocular) and the epipolar line test, the last one at the least
// distance (the reference's "dist > bestDist" skip keeps equal ones coming
// later).  Cw1: pKF1's camera centre; T2: rows 0-2 of pKF2's Tcw; K2: pKF2's
// fx, fy, cx, cy; scale / sigma2: pKF2's mvScaleFactors / mvLevelSigma2.
// match_out[i1]: the pKF2 feature or -1.
int orc_search_for_triangulation(const orc_kp* kps1, const uint8_t* desc1, const uint8_t* mp1, const float* ur1, int n1,
                                  int fv1_n, const int* fv1_nodes, const int* fv1_offsets, const int* fv1_features,
                                  const orc_kp* kps2, const uint8_t* desc2, const uint8_t* mp2, const float* ur2, int n2,
                                  int fv2_n, const int* fv2_nodes, const int* fv2_offsets, const int* fv2_features,
                                  const float* Cw1, const float* T2, const float* K2, const float* F12,
                                  const float* scale, const float* sigma2, int only_stereo, int check_ori,
                                  int* match_out) {
    const int TH_LOW = 50, HISTO = 30;
    (void)n2;
    // the epipole: C2 = R2w * Cw + t2w (double-accumulated product), 1.0f / z
    float C2[3];
    for (int r = 0; r < 3; r++) C2[r] = mat_row_dot(T2 + 4 * r, 1, Cw1) + T2[4 * r + 3];
    const float invz = 1.0f / C2[2];
    const float ex = K2[0] * C2[0] * invz + K2[2];
    const float ey = K2[1] * C2[1] * invz + K2[3];
    std::vector<char> matched2(n2, 0);
    for (int i = 0; i < n1; i++) match_out[i] = -1;
    std::vector<int> hist[HISTO];
    const float factor = HISTO / 360.0f;
    int nmatches = 0, a = 0, b = 0;
    while (a < fv1_n && b < fv2_n) {
        if (fv1_nodes[a] < fv2_nodes[b]) {
            a++;
            continue;
        }
        if (fv1_nodes[a] > fv2_nodes[b]) {
            b++;
            continue;
        }
        for (int p = fv1_offsets[a]; p < fv1_offsets[a + 1]; p++) {
            const int i1 = fv1_features[p];
            if (mp1[i1]) continue;
            const bool st1 = ur1[i1] >= 0;
            if (only_stereo && !st1) continue;
            const orc_kp& k1 = kps1[i1];
            int bestDist = TH_LOW, best2 = -1;
            for (int q = fv2_offsets[b]; q < fv2_offsets[b + 1]; q++) {
                const int i2 = fv2_features[q];
                if (matched2[i2] || mp2[i2]) continue;
                const bool st2 = ur2[i2] >= 0;
                if (only_stereo && !st2) continue;
                const int dist = hamming(desc1 + (size_t)i1 * 32, desc2 + (size_t)i2 * 32);
                if (dist > TH_LOW || dist > bestDist) continue;
                const orc_kp& k2 = kps2[i2];
                if (!st1 && !st2) {
                    const float dx = ex - k2.x, dy = ey - k2.y;
                    if (dx * dx + dy * dy < 100 * scale[k2.octave]) continue;
                }
                // CheckDistEpipolarLine: the line of kp1 in pKF2, distance of kp2 to it
                const float la = k1.x * F12[0] + k1.y * F12[3] + F12[6];
                const float lb = k1.x * F12[1] + k1.y * F12[4] + F12[7];
                const float lc = k1.x * F12[2] + k1.y * F12[5] + F12[8];
                const float num = la * k2.x + lb * k2.y + lc;
                const float den = la * la + lb * lb;
                if (den == 0) continue;
                const float dsqr = num * num / den;
                if (dsqr < 3.84 * sigma2[k2.octave]) {
                    best2 = i2;
                    bestDist = dist;
                }
            }
            if (best2 >= 0) {
                match_out[i1] = best2;
                matched2[best2] = 1;
                nmatches++;
                if (check_ori) {
                    float rot = k1.angle - kps2[best2].angle;
                    if (rot < 0.0) rot += 360.0f;
                    int bin = (int)std::round(rot * factor);
                    if (bin == HISTO) bin = 0;
                    hist[bin].push_back(i1);
                }
            }
        }
        a++;
        b++;
    }
    if (check_ori) {
        int i1 = -1, i2 = -1, i3 = -1;
        three_maxima(hist, HISTO, i1, i2, i3);
        for (int h = 0; h < HISTO; h++) {
            if (h == i1 || h == i2 || h == i3) continue;
            for (int idx1 : hist[h]) {
                matched2[match_out[idx1]] = 0;
                match_out[idx1] = -1;
                nmatches--;
            }
        }
    }
    return nmatches;
}

// ORBmatcher::SearchByProjection(KeyFrame* pKF, Scw, vpPoints, vpMatched,
// th), src/ORBmatcher.cc:423-560: the Sim3 de-scaled (s = sqrt(row 0 . row
// 0), R and t divided by s), depth >= 0, KeyFrame::IsInImage, the distance
// invariance, PO.dot(Pn) >= 0.5 dist, the predicted level, the keyframe's
// window (no level filter) then levels L - 1 .. L, a keypoint of vpMatched
// set (before or during the call) skipped, best <= TH_LOW.  pstate: 1 usable,
// 2 bad.  match_out: >= 0 the point index, -2 claimed before, -1 none.
int orc_search_by_projection_sim3(const orc_params* p, const orc_kp* kps, const uint8_t* desc, int n, int w, int h,
                                  const float* Scw, const float* cam, const orc_mp_geometry* pts,
                                  const uint8_t* pdesc, const uint8_t* pstate, int npts, int th,
                                  const uint8_t* claimed, int* match_out) {
    const Tables t = make_tables(p);
    Grid* g = new Grid();
    build_grid(*g, kps, n, w, h);
    std::vector<int> owner(n);
    for (int i = 0; i < n; i++) owner[i] = (claimed && claimed[i]) ? -2 : -1;
    double d = 0;
    for (int k = 0; k < 3; k++) d += (double)Scw[k] * (double)Scw[k];
    const float scw = (float)std::sqrt(d);
    float T[12];
    for (int k = 0; k < 12; k++) T[k] = Scw[k] / scw;
    const float tcw[3] = {T[3], T[7], T[11]};
    float Ow[3];
    for (int r = 0; r < 3; r++) {
        const float col[3] = {-T[r], -T[4 + r], -T[8 + r]};
        Ow[r] = mat_row_dot(col, 1, tcw);
    }
    const float log_scale = std::log(p->scale_factor);
    int nmatches = 0;
    for (int i = 0; i < npts; i++) {
        if (pstate[i] != 1) continue;
        const orc_mp_geometry& mp = pts[i];
        const float X[3] = {mp.x, mp.y, mp.z};
        float c[3];
        for (int r = 0; r < 3; r++) c[r] = mat_row_dot(T + 4 * r, 1, X) + T[4 * r + 3];
        if (c[2] < 0.0) continue;
        const float invz = 1 / c[2];
        const float x = c[0] * invz, y = c[1] * invz;
        const float u = cam[0] * x + cam[2], v = cam[1] * y + cam[3];
        if (!(u >= 0.0f && u < (float)w && v >= 0.0f && v < (float)h)) continue;
        const float PO[3] = {X[0] - Ow[0], X[1] - Ow[1], X[2] - Ow[2]};
        double ss = 0;
        for (int k = 0; k < 3; k++) ss += (double)PO[k] * (double)PO[k];
        const float dist = (float)std::sqrt(ss);
        if (dist < 0.8f * mp.min_distance || dist > 1.2f * mp.max_distance) continue;
        const double dot = (double)PO[0] * mp.nx + (double)PO[1] * mp.ny + (double)PO[2] * mp.nz;
        if (dot < 0.5 * dist) continue;
        int level = (int)std::ceil(std::log(mp.max_distance / dist) / log_scale);
        if (level < 0) level = 0;
        else if (level >= p->nlevels) level = p->nlevels - 1;
        const float radius = th * t.scale[level];
        const std::vector<int> idx = kf_features_in_area(*g, kps, u, v, radius);
        int bestDist = 256, best = -1;
        for (int k : idx) {
            if (owner[k] != -1) continue;
            if (kps[k].octave < level - 1 || kps[k].octave > level) continue;
            const int dd = hamming(pdesc + (size_t)i * 32, desc + (size_t)k * 32);
            if (dd < bestDist) {
                bestDist = dd;
                best = k;
            }
        }
        if (bestDist <= 50) {
            owner[best] = i;
            nmatches++;
        }
    }
    for (int i = 0; i < n; i++) match_out[i] = owner[i];
    delete g;
    return nmatches;
}

// ORBmatcher::Fuse(KeyFrame*, vpMapPoints, th), src/ORBmatcher.cc:1107-1220,
// the choice of every map point: T rows 0-2 of pKF's pose, cam = fx, fy,
// cx, cy, bf; mp_state 1 usable (2 bad / already in pKF).  target[i]: the
// keyframe feature, or -1.
int orc_fuse_candidates(const orc_params* p, const orc_kp* kps, const uint8_t* desc, const float* uright, int n,
                          int w, int h, const float* T, const float* cam, const orc_mp_geometry* mps,
                          const uint8_t* mp_desc, const uint8_t* mp_state, int m, float th, int* target) {
    const Tables t = make_tables(p);
    Grid* g = new Grid();
    build_grid(*g, kps, n, w, h);
    const float tcw[3] = {T[3], T[7], T[11]};
    float Ow[3];
    for (int r = 0; r < 3; r++) {
        const float col[3] = {-T[r], -T[4 + r], -T[8 + r]};
        Ow[r] = mat_row_dot(col, 1, tcw);
    }
    const float log_scale = std::log(p->scale_factor);
    int nf = 0;
    for (int i = 0; i < m; i++) {
        target[i] = -1;
        if (mp_state[i] != 1) continue;
        const orc_mp_geometry& mp = mps[i];
        const float X[3] = {mp.x, mp.y, mp.z};
        float c[3];
        for (int r = 0; r < 3; r++) c[r] = mat_row_dot(T + 4 * r, 1, X) + T[4 * r + 3];
        if (c[2] < 0.0f) continue;
        const float invz = 1 / c[2];
        const float x = c[0] * invz, y = c[1] * invz;
        const float u = cam[0] * x + cam[2], v = cam[1] * y + cam[3];
        if (!(u >= 0.0f && u < (float)w && v >= 0.0f && v < (float)h)) continue;
        const float ur = u - cam[4] * invz;
        const float PO[3] = {X[0] - Ow[0], X[1] - Ow[1], X[2] - Ow[2]};
        double ss = 0;
        for (int k = 0; k < 3; k++) ss += (double)PO[k] * (double)PO[k];
        const float dist3D = (float)std::sqrt(ss);
        if (dist3D < 0.8f * mp.min_distance || dist3D > 1.2f * mp.max_distance) continue;
        const double dot = (double)PO[0] * mp.nx + (double)PO[1] * mp.ny + (double)PO[2] * mp.nz;
        if (dot < 0.5 * dist3D) continue;
        int level = (int)std::ceil(std::log(mp.max_distance / dist3D) / log_scale);
        if (level < 0) level = 0;
        else if (level >= p->nlevels) level = p->nlevels - 1;
        const float radius = th * t.scale[level];
        const std::vector<int> idx = kf_features_in_area(*g, kps, u, v, radius);
        int bestDist = 256, best = -1;
        for (int k : idx) {
            const int kl = kps[k].octave;
            if (kl < level - 1 || kl > level) continue;
            const float ex = u - kps[k].x, ey = v - kps[k].y;
            if (uright && uright[k] >= 0) {
                const float er = ur - uright[k];
                const float e2 = ex * ex + ey * ey + er * er;
                if (e2 * t.inv_sigma2[kl] > 7.8) continue;
            } else {
                const float e2 = ex * ex + ey * ey;
                if (e2 * t.inv_sigma2[kl] > 5.99) continue;
            }
            const int dd = hamming(mp_desc + (size_t)i * 32, desc + (size_t)k * 32);
            if (dd < bestDist) {
                bestDist = dd;
                best = k;
            }
        }
        if (bestDist <= 50) {
            target[i] = best;
            nf++;
        }
    }
    delete g;
    return nf;
}

// ORBmatcher::Fuse(KeyFrame*, Scw, vpPoints, th, vpReplacePoint),
// src/ORBmatcher.cc:1290-1380, the choice of every point: the de-scaled Sim3,
// invz = 1.0 / z (double), no reprojection gate; pstate 1 usable.
int orc_fuse_sim3_candidates(const orc_params* p, const orc_kp* kps, const uint8_t* desc, int n, int w, int h,
                               const float* Scw, const float* cam, const orc_mp_geometry* pts, const uint8_t* pdesc,
                               const uint8_t* pstate, int npts, float th, int* target) {
    const Tables t = make_tables(p);
    Grid* g = new Grid();
    build_grid(*g, kps, n, w, h);
    double d = 0;
    for (int k = 0; k < 3; k++) d += (double)Scw[k] * (double)Scw[k];
    const float scw = (float)std::sqrt(d);
    float T[12];
    for (int k = 0; k < 12; k++) T[k] = Scw[k] / scw;
    const float tcw[3] = {T[3], T[7], T[11]};
    float Ow[3];
    for (int r = 0; r < 3; r++) {
        const float col[3] = {-T[r], -T[4 + r], -T[8 + r]};
        Ow[r] = mat_row_dot(col, 1, tcw);
    }
    const float log_scale = std::log(p->scale_factor);
    int nf = 0;
    for (int i = 0; i < npts; i++) {
        target[i] = -1;
        if (pstate[i] != 1) continue;
        const orc_mp_geometry& mp = pts[i];
        const float X[3] = {mp.x, mp.y, mp.z};
        float c[3];
        for (int r = 0; r < 3; r++) c[r] = mat_row_dot(T + 4 * r, 1, X) + T[4 * r + 3];
        if (c[2] < 0.0f) continue;
        const float invz = 1.0 / c[2];
        const float x = c[0] * invz, y = c[1] * invz;
        const float u = cam[0] * x + cam[2], v = cam[1] * y + cam[3];
        if (!(u >= 0.0f && u < (float)w && v >= 0.0f && v < (float)h)) continue;
        const float PO[3] = {X[0] - Ow[0], X[1] - Ow[1], X[2] - Ow[2]};
        double ss = 0;
        for (int k = 0; k < 3; k++) ss += (double)PO[k] * (double)PO[k];
        const float dist3D = (float)std::sqrt(ss);
        if (dist3D < 0.8f * mp.min_distance || dist3D > 1.2f * mp.max_distance) continue;
        const double dot = (double)PO[0] * mp.nx + (double)PO[1] * mp.ny + (double)PO[2] * mp.nz;
        if (dot < 0.5 * dist3D) continue;
        int level = (int)std::ceil(std::log(mp.max_distance / dist3D) / log_scale);
        if (level < 0) level = 0;
        else if (level >= p->nlevels) level = p->nlevels - 1;
        const float radius = th * t.scale[level];
        const std::vector<int> idx = kf_features_in_area(*g, kps, u, v, radius);
        int bestDist = INT_MAX, best = -1;
        for (int k : idx) {
            if (kps[k].octave < level - 1 || kps[k].octave > level) continue;
            const int dd = hamming(pdesc + (size_t)i * 32, desc + (size_t)k * 32);
            if (dd < bestDist) {
                bestDist = dd;
                best = k;
            }
        }
        if (bestDist <= 50) {
            target[i] = best;
            nf++;
        }
    }
    delete g;
    return nf;
}

// ORBmatcher::SearchBySim3(pKF1, pKF2, vpMatches12, s12, R12, t12, th),
// src/ORBmatcher.cc:1441-1640 (vpMatches12 empty on entry): pKF1's map points
// through R1w, t1w then sR21 = (1/s12) R12^T, t21 = -sR21 t12 into pKF2 and
// pKF2's through R2w, t2w then sR12 = s12 R12, t12 into pKF1, each the first
// least distance <= TH_HIGH in its window (levels predicted - 1 .. predicted,
// depth |p3Dc|, pKF1's camera for both); kept where both agree.  st: 1 usable.
static int sim3_side(const Tables& t, const Grid& g, const orc_kp* kps, const uint8_t* desc, int w, int h,
                     const float* Tw, const float* sR, const float* tt, const float* cam, float log_scale,
                     int nlevels, const orc_mp_geometry& mp, const uint8_t* mpd, float th) {
    const float X[3] = {mp.x, mp.y, mp.z};
    float c1[3], c2[3];
    for (int r = 0; r < 3; r++) c1[r] = mat_row_dot(Tw + 4 * r, 1, X) + Tw[4 * r + 3];
    for (int r = 0; r < 3; r++) c2[r] = mat_row_dot(sR + 3 * r, 1, c1) + tt[r];
    if (c2[2] < 0.0) return -1;
    const float invz = 1.0 / c2[2];
    const float x = c2[0] * invz, y = c2[1] * invz;
    const float u = cam[0] * x + cam[2], v = cam[1] * y + cam[3];
    if (!(u >= 0.0f && u < (float)w && v >= 0.0f && v < (float)h)) return -1;
    double ss = 0;
    for (int k = 0; k < 3; k++) ss += (double)c2[k] * (double)c2[k];
    const float dist3D = (float)std::sqrt(ss);
    if (dist3D < 0.8f * mp.min_distance || dist3D > 1.2f * mp.max_distance) return -1;
    int level = (int)std::ceil(std::log(mp.max_distance / dist3D) / log_scale);
    if (level < 0) level = 0;
    else if (level >= nlevels) level = nlevels - 1;
    const float radius = th * t.scale[level];
    const std::vector<int> idx = kf_features_in_area(g, kps, u, v, radius);
    int bestDist = INT_MAX, best = -1;
    for (int k : idx) {
        if (kps[k].octave < level - 1 || kps[k].octave > level) continue;
        const int dd = hamming(mpd, desc + (size_t)k * 32);
        if (dd < bestDist) {
            bestDist = dd;
            best = k;
        }
    }
    return bestDist <= kThHigh ? best : -1;
}

int orc_search_by_sim3(const orc_params* p, const orc_kp* kps1, const uint8_t* desc1, int n1, const orc_kp* kps2,
                           const uint8_t* desc2, int n2, int w, int h, const float* T1w, const float* T2w, float s12,
                           const float* R12, const float* t12, const float* cam, const orc_mp_geometry* mps1,
                           const uint8_t* mpd1, const uint8_t* st1, const orc_mp_geometry* mps2, const uint8_t* mpd2,
                           const uint8_t* st2, float th, int* match12) {
    const Tables t = make_tables(p);
    Grid* g1 = new Grid();
    Grid* g2 = new Grid();
    build_grid(*g1, kps1, n1, w, h);
    build_grid(*g2, kps2, n2, w, h);
    float sR12[9], sR21[9], nsR21[9], t21[3];
    const float inv_s = (float)(1.0 / (double)s12);
    for (int r = 0; r < 3; r++)
        for (int c = 0; c < 3; c++) {
            sR12[3 * r + c] = R12[3 * r + c] * s12;
            sR21[3 * r + c] = R12[3 * c + r] * inv_s;
            nsR21[3 * r + c] = -sR21[3 * r + c];
        }
    for (int r = 0; r < 3; r++) t21[r] = mat_row_dot(nsR21 + 3 * r, 1, t12);
    const float log_scale = std::log(p->scale_factor);
    std::vector<int> m1(n1, -1), m2(n2, -1);
    for (int i = 0; i < n1; i++)
        if (st1[i] == 1)
            m1[i] = sim3_side(t, *g2, kps2, desc2, w, h, T1w, sR21, t21, cam, log_scale, p->nlevels, mps1[i],
                              mpd1 + (size_t)i * 32, th);
    for (int i = 0; i < n2; i++)
        if (st2[i] == 1)
            m2[i] = sim3_side(t, *g1, kps1, desc1, w, h, T2w, sR12, t12, cam, log_scale, p->nlevels, mps2[i],
                              mpd2 + (size_t)i * 32, th);
    int found = 0;
    for (int i = 0; i < n1; i++) {
        match12[i] = (m1[i] >= 0 && m2[m1[i]] == i) ? m1[i] : -1;
        found += match12[i] >= 0;
    }
    delete g1;
    delete g2;
    return found;
}

// Frame::ComputeStereoMatches, src/Frame.cc:831-1082 (mb = mbf/fx).
int orc_compute_stereo_matches(const orc_params* p, const orc_kp* kpsL, const uint8_t* descL, int nL,
                               const orc_kp* kpsR, const uint8_t* descR, int nR, const uint8_t* pyrL,
                               const uint8_t* pyrR, const int* level_w, const int* level_h, int w, int h, float bf,
                               float fx, float* uright, float* depth) {
    (void)w;
    const Tables t = make_tables(p);
    std::vector<size_t> off(p->nlevels, 0);
    for (int l = 1; l < p->nlevels; l++) off[l] = off[l - 1] + (size_t)level_w[l - 1] * level_h[l - 1];
    for (int i = 0; i < nL; i++) uright[i] = depth[i] = -1.0f;
    const int thOrbDist = (kThHigh + kThLow) / 2;
    const int nRows = level_h[0];
    (void)h;
    std::vector<std::vector<int> > rows(nRows);
    for (int iR = 0; iR < nR; iR++) {
        const float kpY = kpsR[iR].y;
        const float r = 2.0f * t.scale[kpsR[iR].octave];
        const int maxr = (int)std::ceil(kpY + r), minr = (int)std::floor(kpY - r);
        for (int yi = minr; yi <= maxr; yi++) rows[yi].push_back(iR);
    }
    const float mb = bf / fx;
    const float minZ = mb, minD = 0, maxD = bf / minZ;
    std::vector<std::pair<int, int> > distIdx;
    for (int iL = 0; iL < nL; iL++) {
        const orc_kp& kpL = kpsL[iL];
        const int levelL = kpL.octave;
        const float vL = kpL.y, uL = kpL.x;
        const std::vector<int>& cands = rows[(size_t)vL];
        if (cands.empty()) continue;
        const float minU = uL - maxD, maxU = uL - minD;
        if (maxU < 0) continue;
        int bestDist = kThHigh;
        int bestIdxR = 0;
        for (int iR : cands) {
            const orc_kp& kpR = kpsR[iR];
            if (kpR.octave < levelL - 1 || kpR.octave > levelL + 1) continue;
            const float uR = kpR.x;
            if (uR >= minU && uR <= maxU) {
                const int dist = hamming(descL + (size_t)iL * 32, descR + (size_t)iR * 32);
                if (dist < bestDist) {
                    bestDist = dist;
                    bestIdxR = iR;
                }
            }
        }
        if (bestDist >= thOrbDist) continue;
        const float uR0 = kpsR[bestIdxR].x;
        const float sf = t.inv_scale[levelL];
        const float scaleduL = std::round(kpL.x * sf), scaledvL = std::round(kpL.y * sf);
        const float scaleduR0 = std::round(uR0 * sf);
        const int W = 5, L = 5;
        const int lw = level_w[levelL];
        const uint8_t* left = pyrL + off[levelL];
        const uint8_t* right = pyrR + off[levelL];
        const int ly0 = (int)(scaledvL - W), lx0 = (int)(scaleduL - W);
        const float cl = (float)left[(size_t)(ly0 + W) * lw + lx0 + W];
        const float iniu = scaleduR0 - L - W, endu = scaleduR0 + L + W + 1;
        if (iniu < 0 || endu >= lw) continue;
        int bestSad = INT_MAX, bestincR = 0;
        float dists[2 * L + 1];
        for (int incR = -L; incR <= L; incR++) {
            const int rx0 = (int)(scaleduR0 + incR - W);
            const float cr = (float)right[(size_t)(ly0 + W) * lw + rx0 + W];
            double s = 0;
            for (int yy = 0; yy < 2 * W + 1; yy++)
                for (int xx = 0; xx < 2 * W + 1; xx++) {
                    const float a = (float)left[(size_t)(ly0 + yy) * lw + lx0 + xx] - cl;
                    const float b = (float)right[(size_t)(ly0 + yy) * lw + rx0 + xx] - cr;
                    s += std::fabs((double)(a - b));
                }
            const float dist = (float)s;
            if (dist < bestSad) {
                bestSad = (int)dist;
                bestincR = incR;
            }
            dists[L + incR] = dist;
        }
        if (bestincR == -L || bestincR == L) continue;
        const float d1 = dists[L + bestincR - 1], d2 = dists[L + bestincR], d3 = dists[L + bestincR + 1];
        const float deltaR = (d1 - d3) / (2.0f * (d1 + d3 - 2.0f * d2));
        if (deltaR < -1 || deltaR > 1) continue;
        float bestuR = t.scale[levelL] * ((float)scaleduR0 + (float)bestincR + deltaR);
        float disparity = uL - bestuR;
        if (disparity >= minD && disparity < maxD) {
            if (disparity <= 0) {
                disparity = 0.01;
                bestuR = uL - 0.01;
            }
            depth[iL] = bf / disparity;
            uright[iL] = bestuR;
            distIdx.push_back(std::make_pair(bestSad, iL));
        }
    }
    if (distIdx.empty()) return 0;
    std::sort(distIdx.begin(), distIdx.end());
    const float median = distIdx[distIdx.size() / 2].first;
    const float thDist = 1.5f * 1.4f * median;
    for (int i = (int)distIdx.size() - 1; i >= 0; i--) {
        if (distIdx[i].first < thDist) break;
        uright[distIdx[i].second] = -1;
        depth[distIdx[i].second] = -1;
    }
    return (int)distIdx.size();
}

int orc_knn2(const uint8_t* q, int nq, const uint8_t* t, int nt, int* idx1, int* d1, int* idx2, int* d2) {
    for (int i = 0; i < nq; i++) {
        int b1 = INT_MAX, b2 = INT_MAX, i1 = -1, i2 = -1;
        for (int j = 0; j < nt; j++) {
            const int d = hamming(q + (size_t)i * 32, t + (size_t)j * 32);
            if (d < b1) {
                b2 = b1; i2 = i1; b1 = d; i1 = j;
            } else if (d < b2) {
                b2 = d; i2 = j;
            }
        }
        idx1[i] = i1; d1[i] = b1; idx2[i] = i2; d2[i] = b2;
    }
    return 0;
}

void orc_blur_level(const uint8_t* src, int w, int h, uint8_t* dst) { shim_gauss7_u8(src, w, w, h, dst, w); }

int orc_fast_level(const uint8_t* level, int w, int h, int ini_th, int min_th, orc_kp* out, int cap) {
    Level L;
    L.w = w;
    L.h = h;
    L.px.assign(level, level + (size_t)w * h);
    std::vector<orc_kp> v = fast_level(L, ini_th, min_th);
    for (int i = 0; i < (int)v.size() && i < cap; i++) out[i] = v[i];
    return (int)v.size();
}

int orc_distribute(const orc_kp* cand, int n, int minX, int maxX, int minY, int maxY, int N, orc_kp* out, int cap) {
    std::vector<orc_kp> c(cand, cand + n);
    std::vector<orc_kp> r = distribute(c, minX, maxX, minY, maxY, N);
    for (int i = 0; i < (int)r.size() && i < cap; i++) out[i] = r[i];
    return (int)r.size();
}

// cv::undistortPoints(src, dst, K, dist, noArray(), K) as Frame calls it,
// restated from OpenCV 3.2's cvUndistortPoints: normalise by the camera
// matrix in double, 5 rounds of x = (x0 - tangential) / radial, back through
// K, rounded to float.  k = k1 k2 p1 p2 k3 (k3 = 0 for four coefficients).
static void undistort_point(double fx, double fy, double cx, double cy, const double* k, float& u, float& v) {
    const double ifx = 1. / fx, ify = 1. / fy;
    const double x0 = (u - cx) * ifx, y0 = (v - cy) * ify;
    double x = x0, y = y0;
    for (int it = 0; it < 5; it++) {
        const double r2 = x * x + y * y;
        const double radial = 1 + ((k[4] * r2 + k[1]) * r2 + k[0]) * r2;
        const double icdist = 1 / radial;
        const double dx = 2 * k[2] * x * y + k[3] * (r2 + 2 * x * x);
        const double dy = k[2] * (r2 + 2 * y * y) + 2 * k[3] * x * y;
        x = (x0 - dx) * icdist;
        y = (y0 - dy) * icdist;
    }
    u = (float)(fx * x + 0.0 * y + cx);
    v = (float)(0.0 * x + fy * y + cy);
}

// Frame::UndistortKeyPoints, src/Frame.cc:724-776: nothing to do when the
// first coefficient is zero (whatever the others), else every keypoint
// through undistort_point (the other keypoint fields are copied).
int orc_undistort_keypoints(const float* K4, const float* dist, int ndist, const orc_kp* kps, int n, orc_kp* out) {
    double k[5] = {0, 0, 0, 0, 0};
    for (int i = 0; i < ndist && i < 5; i++) k[i] = dist[i];
    for (int i = 0; i < n; i++) {
        out[i] = kps[i];
        if (dist[0] != 0.0f) undistort_point(K4[0], K4[1], K4[2], K4[3], k, out[i].x, out[i].y);
    }
    return 0;
}

// Frame::ComputeImageBounds, src/Frame.cc:778-819: the undistorted corners
// give min over the left / top pair and max over the right / bottom pair.
int orc_compute_image_bounds(int cols, int rows, const float* K4, const float* dist, int ndist, float* bounds) {
    if (dist[0] == 0.0f) {
        bounds[0] = 0.0f;
        bounds[1] = (float)cols;
        bounds[2] = 0.0f;
        bounds[3] = (float)rows;
        return 0;
    }
    double k[5] = {0, 0, 0, 0, 0};
    for (int i = 0; i < ndist && i < 5; i++) k[i] = dist[i];
    float cx[4] = {0.0f, (float)cols, 0.0f, (float)cols}, cy[4] = {0.0f, 0.0f, (float)rows, (float)rows};
    for (int c = 0; c < 4; c++) undistort_point(K4[0], K4[1], K4[2], K4[3], k, cx[c], cy[c]);
    bounds[0] = std::min(cx[0], cx[2]);
    bounds[1] = std::max(cx[1], cx[3]);
    bounds[2] = std::min(cy[0], cy[1]);
    bounds[3] = std::max(cy[2], cy[3]);
    return 0;
}

// Frame::isInFrustum, src/Frame.cc:491-578, as the reference computes it
// against the cv stand-in: the pose matrices of Frame::UpdatePoseMatrices
// (:454-470; mOw = -mRcw^T mtcw), Pc = mRcw * P + mtcw with the product
// accumulated in double and rounded to float before the float add, the
// projection and bounds in float, GetMin/MaxDistanceInvariance (0.8f / 1.2f
// times the stored distances, src/MapPoint.cc:542-552), dist = cv::norm(P -
// mOw) (double sum of squares, double sqrt, to float), viewCos = PO.dot(Pn)
// (double) / dist, and MapPoint::PredictScale(dist, Frame*)
// (src/MapPoint.cc:604-619): ceil(logf(mfMaxDistance / dist) /
// logf(mfScaleFactor)) clamped to [0, nlevels - 1].
int orc_is_in_frustum(const orc_frustum_camera* cam, const orc_mp_geometry* mps, int m, float cos_limit,
                      orc_mappoint* out) {
    float R[3][3], t[3], Ow[3];
    for (int r = 0; r < 3; r++) {
        for (int c = 0; c < 3; c++) R[r][c] = cam->Tcw[4 * r + c];
        t[r] = cam->Tcw[4 * r + 3];
    }
    for (int i = 0; i < 3; i++) {
        double s = 0;
        for (int k = 0; k < 3; k++) s += (double)(-R[k][i]) * (double)t[k];
        Ow[i] = (float)s;
    }
    const float log_scale = std::log(cam->scale_factor);
    int nin = 0;
    for (int i = 0; i < m; i++) {
        const orc_mp_geometry& g = mps[i];
        orc_mappoint& o = out[i];
        o.track_in_view = 0;
        const float P[3] = {g.x, g.y, g.z};
        float Pc[3];
        for (int r = 0; r < 3; r++) {
            double s = 0;
            for (int k = 0; k < 3; k++) s += (double)R[r][k] * (double)P[k];
            Pc[r] = (float)s + t[r];
        }
        if (Pc[2] < 0.0f) continue;
        const float invz = 1.0f / Pc[2];
        const float u = cam->fx * Pc[0] * invz + cam->cx;
        const float v = cam->fy * Pc[1] * invz + cam->cy;
        if (u < cam->min_x || u > cam->max_x) continue;
        if (v < cam->min_y || v > cam->max_y) continue;
        const float max_d = 1.2f * g.max_distance;
        const float min_d = 0.8f * g.min_distance;
        const float PO[3] = {P[0] - Ow[0], P[1] - Ow[1], P[2] - Ow[2]};
        double ss = 0;
        for (int k = 0; k < 3; k++) ss += (double)PO[k] * (double)PO[k];
        const float dist = (float)std::sqrt(ss);
        if (dist < min_d || dist > max_d) continue;
        const double dot = (double)PO[0] * g.nx + (double)PO[1] * g.ny + (double)PO[2] * g.nz;
        const float view_cos = (float)(dot / dist);
        if (view_cos < cos_limit) continue;
        const float ratio = g.max_distance / dist;
        int level = (int)std::ceil(std::log(ratio) / log_scale);
        if (level < 0) level = 0;
        else if (level >= cam->nlevels) level = cam->nlevels - 1;
        o.track_in_view = 1;
        o.proj_x = u;
        o.proj_xr = u - cam->bf * invz;
        o.proj_y = v;
        o.track_scale_level = level;
        o.view_cos = view_cos;
        nin++;
    }
    return nin;
}

// ---------------------------------------------------------------- DBoW2
// The vocabulary tree of Thirdparty/DBoW2/DBoW2/TemplatedVocabulary.h as
// loadFromTextFile (:1368-1460) builds it: node 0 the root, then one node per
// line in file order ("parent is_leaf d0 .. d31 weight"), appended to its
// parent's children; leaves (by the file flag) numbered as words in file
// order.  The descent stops at a node without children (Node::isLeaf).
namespace {
struct OrcVocab {
    int k = 0, L = 0, scoring = 0, weighting = 0, nwords = 0;
    std::vector<std::vector<int> > children;
    std::vector<std::array<uint8_t, 32> > desc;
    std::vector<double> weight;
    std::vector<int> word_id;
};
std::map<std::string, OrcVocab> g_vocabs;

bool load_vocab(const std::string& path, OrcVocab& v) {
    std::ifstream f(path.c_str());
    if (!f.is_open()) return false;
    std::string line;
    if (!std::getline(f, line)) return false;
    std::stringstream hs(line);
    int n1 = -1, n2 = -1;
    hs >> v.k >> v.L >> n1 >> n2;
    if (v.k < 0 || v.k > 20 || v.L < 1 || v.L > 10 || n1 < 0 || n1 > 5 || n2 < 0 || n2 > 3) return false;
    v.scoring = n1;
    v.weighting = n2;
    v.children.assign(1, std::vector<int>());
    v.desc.assign(1, std::array<uint8_t, 32>());
    v.weight.assign(1, 0.0);
    v.word_id.assign(1, 0);
    while (std::getline(f, line)) {
        if (line.empty()) return false;  // the reference would append a node of unset bytes
        std::stringstream ls(line);
        const int nid = (int)v.children.size();
        int pid = -1, leaf = 0;
        ls >> pid >> leaf;
        if (ls.fail() || pid < 0 || pid >= nid) return false;
        std::array<uint8_t, 32> d;
        for (int i = 0; i < 32; i++) {
            int b = 0;
            ls >> b;
            d[i] = (uint8_t)b;
        }
        double w = 0;
        ls >> w;
        if (ls.fail()) return false;
        v.children.push_back(std::vector<int>());
        v.children[pid].push_back(nid);
        v.desc.push_back(d);
        v.weight.push_back(w);
        v.word_id.push_back(leaf > 0 ? v.nwords++ : 0);
    }
    return true;
}

// TemplatedVocabulary::transform(feature, word_id, weight, nid, levelsup),
// TemplatedVocabulary.h:1240-1290: from the root, the first child with the
// least distance at every level (strict <), the node of level L - levelsup
// kept for the feature vector (the root when that level is <= 0).
void vocab_descend(const OrcVocab& v, const uint8_t* f, int levelsup, int& word, double& weight, int& nid) {
    const int nid_level = v.L - levelsup;
    nid = 0;
    int node = 0, level = 0;
    do {
        ++level;
        const std::vector<int>& ch = v.children[node];
        int best = ch[0];
        int best_d = hamming(f, v.desc[best].data());
        for (size_t c = 1; c < ch.size(); c++) {
            const int d = hamming(f, v.desc[ch[c]].data());
            if (d < best_d) {
                best_d = d;
                best = ch[c];
            }
        }
        node = best;
        if (level == nid_level) nid = node;
    } while (!v.children[node].empty());
    word = v.word_id[node];
    weight = v.weight[node];
}
}  // namespace

extern "C" {

// The same tree from arrays (entry i describes node i + 1), stored under a
// name usable as the path argument of orc_bow_transform.
int orc_vocabulary_from_arrays(const char* name, int k, int L, int scoring, int weighting, int nnodes,
                               const int* parents, const uint8_t* is_leaf, const uint8_t* descriptors,
                               const double* weights) {
    OrcVocab v;
    v.k = k;
    v.L = L;
    v.scoring = scoring;
    v.weighting = weighting;
    v.children.assign(nnodes, std::vector<int>());
    v.desc.assign(nnodes, std::array<uint8_t, 32>());
    v.weight.assign(nnodes, 0.0);
    v.word_id.assign(nnodes, 0);
    for (int i = 0; i + 1 < nnodes; i++) {
        const int node = i + 1;
        if (parents[i] < 0 || parents[i] > i) return -1;
        v.children[parents[i]].push_back(node);
        std::memcpy(v.desc[node].data(), descriptors + (size_t)i * 32, 32);
        v.weight[node] = weights[i];
        v.word_id[node] = is_leaf[i] ? v.nwords++ : 0;
    }
    g_vocabs[name] = v;
    return v.nwords;
}

int orc_vocabulary_load(const char* path) {
    OrcVocab v;
    if (!load_vocab(path, v)) return -1;
    g_vocabs[path] = v;
    return v.nwords;
}

// TemplatedVocabulary::transform(features, BowVector, FeatureVector,
// levelsup), TemplatedVocabulary.h:1136-1205, with BowVector::addWeight /
// addIfNotExist / normalize (BowVector.cpp:40-95) and
// FeatureVector::addFeature (FeatureVector.cpp:37-53), as Frame::ComputeBoW
// (src/Frame.cc:704-718) calls it with levelsup 4.  Per feature: word, weight
// and feature-vector node.  BowVector: bow_n (word, value) pairs in ascending
// word order.  FeatureVector: fv_n nodes in ascending order, node i owning
// fv_features[fv_offsets[i] .. fv_offsets[i + 1]) in feature order.
int orc_bow_transform(const char* path, const uint8_t* desc, int n, int levelsup, int* word_ids, double* weights,
                      int* node_ids, int* bow_n, int* bow_words, double* bow_values, int* fv_n, int* fv_nodes,
                      int* fv_offsets, int* fv_features) {
    auto it = g_vocabs.find(path);
    if (it == g_vocabs.end()) return -1;
    const OrcVocab& v = it->second;
    std::map<int, double> bow;
    std::map<int, std::vector<int> > fv;
    if (v.nwords > 0) {
        const bool tf = v.weighting == 0 || v.weighting == 1;  // TF_IDF, TF
        for (int i = 0; i < n; i++) {
            int w_id, nid;
            double w;
            vocab_descend(v, desc + (size_t)i * 32, levelsup, w_id, w, nid);
            word_ids[i] = w_id;
            weights[i] = w;
            node_ids[i] = nid;
            if (!(w > 0)) continue;
            auto b = bow.find(w_id);
            if (b == bow.end()) bow[w_id] = w;
            else if (tf) b->second += w;
            fv[nid].push_back(i);
        }
        // L1 for L1 / chi-square / KL / Bhattacharyya, L2 for L2, none for
        // the dot product (ScoringObject.h:84-89)
        const bool must = v.scoring != 5;
        if (tf && !bow.empty() && !must) {
            const double nd = (double)bow.size();
            for (auto& e : bow) e.second /= nd;
        }
        if (must) {
            double norm = 0.0;
            if (v.scoring != 1) {
                for (auto& e : bow) norm += std::fabs(e.second);
            } else {
                for (auto& e : bow) norm += e.second * e.second;
                norm = std::sqrt(norm);
            }
            if (norm > 0.0)
                for (auto& e : bow) e.second /= norm;
        }
    } else {
        for (int i = 0; i < n; i++) word_ids[i] = node_ids[i] = -1, weights[i] = 0.0;
    }
    int b = 0;
    for (auto& e : bow) {
        bow_words[b] = e.first;
        bow_values[b] = e.second;
        b++;
    }
    *bow_n = b;
    int nn = 0, off = 0;
    for (auto& e : fv) {
        fv_nodes[nn] = e.first;
        fv_offsets[nn] = off;
        for (int f : e.second) fv_features[off++] = f;
        nn++;
    }
    fv_offsets[nn] = off;
    *fv_n = nn;
    return 0;
}

}  // extern "C"

// ORBmatcher::SearchByBoW(KeyFrame* pKF, Frame& F, vpMapPointMatches),
// src/ORBmatcher.cc:247-380: the nodes both FeatureVectors hold, in ascending
// order; in a node every keyframe feature with a map point that is not bad
// (in list order) takes the frame feature of the node, not yet matched, at
// the least distance (first in list order; second-best over the rest); kept
// when best <= TH_LOW and best < nnratio * second; then the rotation check
// (three_maxima).  kf_mp: 0 no map point, 1 a map point, 2 a bad one.
// match_out[i]: the keyframe feature whose map point frame feature i got, or -1.
// keyframes: SearchByBoW(KeyFrame* pKF1, KeyFrame* pKF2, vpMatches12),
// src/ORBmatcher.cc:729-880 -- candidates need a map point that is not bad
// (f_mp), TH_LOW is exclusive, the result is per pKF1 feature.
static int search_by_bow_impl(const orc_kp* kf_kps, const uint8_t* kf_desc, const uint8_t* kf_mp, int kf_n,
                              int kf_fv_n, const int* kf_fv_nodes, const int* kf_fv_offsets,
                              const int* kf_fv_features, const orc_kp* f_kps, const uint8_t* f_desc,
                              const uint8_t* f_mp, int f_n, int f_fv_n, const int* f_fv_nodes,
                              const int* f_fv_offsets, const int* f_fv_features, float nnratio, int check_ori,
                              bool keyframes, int* match_out) {
    const int TH_LOW = 50, HISTO = 30;
    const int nout = keyframes ? kf_n : f_n;
    for (int i = 0; i < nout; i++) match_out[i] = -1;
    std::vector<char> taken(f_n, 0);
    std::vector<int> hist[HISTO];
    const float factor = HISTO / 360.0f;
    int nmatches = 0;
    int a = 0, b = 0;
    while (a < kf_fv_n && b < f_fv_n) {
        if (kf_fv_nodes[a] < f_fv_nodes[b]) {
            a++;
            continue;
        }
        if (kf_fv_nodes[a] > f_fv_nodes[b]) {
            b++;
            continue;
        }
        for (int p = kf_fv_offsets[a]; p < kf_fv_offsets[a + 1]; p++) {
            const int ikf = kf_fv_features[p];
            if (kf_mp[ikf] != 1) continue;
            int best1 = 256, best2 = 256, bestIdx = -1;
            for (int q = f_fv_offsets[b]; q < f_fv_offsets[b + 1]; q++) {
                const int jf = f_fv_features[q];
                if (taken[jf] || (keyframes && f_mp[jf] != 1)) continue;
                const int d = hamming(kf_desc + (size_t)ikf * 32, f_desc + (size_t)jf * 32);
                if (d < best1) {
                    best2 = best1;
                    best1 = d;
                    bestIdx = jf;
                } else if (d < best2) {
                    best2 = d;
                }
            }
            if ((keyframes ? best1 < TH_LOW : best1 <= TH_LOW) && (float)best1 < nnratio * (float)best2) {
                taken[bestIdx] = 1;
                const int slot = keyframes ? ikf : bestIdx;
                match_out[slot] = keyframes ? bestIdx : ikf;
                if (check_ori) {
                    float rot = kf_kps[ikf].angle - f_kps[bestIdx].angle;
                    if (rot < 0.0) rot += 360.0f;
                    int bin = (int)std::round(rot * factor);
                    if (bin == HISTO) bin = 0;
                    hist[bin].push_back(slot);
                }
                nmatches++;
            }
        }
        a++;
        b++;
    }
    if (check_ori) {
        int i1 = -1, i2 = -1, i3 = -1;
        three_maxima(hist, HISTO, i1, i2, i3);
        for (int h = 0; h < HISTO; h++) {
            if (h == i1 || h == i2 || h == i3) continue;
            for (int slot : hist[h]) {
                match_out[slot] = -1;
                nmatches--;
            }
        }
    }
    return nmatches;
}

int orc_search_by_bow(const orc_kp* kf_kps, const uint8_t* kf_desc, const uint8_t* kf_mp, int kf_n, int kf_fv_n,
                      const int* kf_fv_nodes, const int* kf_fv_offsets, const int* kf_fv_features, const orc_kp* f_kps,
                      const uint8_t* f_desc, int f_n, int f_fv_n, const int* f_fv_nodes, const int* f_fv_offsets,
                      const int* f_fv_features, float nnratio, int check_ori, int* match_out) {
    return search_by_bow_impl(kf_kps, kf_desc, kf_mp, kf_n, kf_fv_n, kf_fv_nodes, kf_fv_offsets, kf_fv_features,
                              f_kps, f_desc, nullptr, f_n, f_fv_n, f_fv_nodes, f_fv_offsets, f_fv_features, nnratio,
                              check_ori, false, match_out);
}

int orc_search_by_bow_kf(const orc_kp* kps1, const uint8_t* desc1, const uint8_t* mp1, int n1, int fv1_n,
                         const int* fv1_nodes, const int* fv1_offsets, const int* fv1_features, const orc_kp* kps2,
                         const uint8_t* desc2, const uint8_t* mp2, int n2, int fv2_n, const int* fv2_nodes,
                         const int* fv2_offsets, const int* fv2_features, float nnratio, int check_ori,
                         int* match_out) {
    return search_by_bow_impl(kps1, desc1, mp1, n1, fv1_n, fv1_nodes, fv1_offsets, fv1_features, kps2, desc2, mp2,
                              n2, fv2_n, fv2_nodes, fv2_offsets, fv2_features, nnratio, check_ori, true, match_out);
}

// MapPoint::PredictScale(currentDist, Frame*), src/MapPoint.cc:604-619, on
// given ratios mfMaxDistance / currentDist.
void orc_predict_scale(const float* ratio, int n, float scale_factor, int nlevels, int* out) {
    const float log_scale = std::log(scale_factor);
    for (int i = 0; i < n; i++) {
        int level = (int)std::ceil(std::log(ratio[i]) / log_scale);
        if (level < 0) level = 0;
        else if (level >= nlevels) level = nlevels - 1;
        out[i] = level;
    }
}

// MapPoint::ComputeDistinctiveDescriptors, src/MapPoint.cc:365-447, for m
// map points given as ragged lists of pool rows in observation order (the
// iteration order of MapPoint::mObservations).  A row of -1 stands for an
// observation whose keyframe is bad (skipped at :391-394).  The reference
// collects the valid descriptors, fills the symmetric N x N table of
// DescriptorDistance values (:403-420), sorts each row, takes element
// (size_t)(0.5 * (N - 1)) as that descriptor's median (:427-434) and keeps
// the first descriptor with the least median (:437-441, strict <).
// best_rows[i] = the chosen pool row, -1 when no observation is valid (the
// reference returns early and leaves mDescriptor as it was), -2 for an
// invalid list (a row outside [-1, pool_rows) or a decreasing offset).
// desc_inout (nullable) receives the chosen row's 32 bytes where
// best_rows[i] >= 0 and is left unchanged elsewhere.
int orc_distinctive_descriptors(const uint8_t* pool, int pool_rows, const int* offsets, const int* rows, int m,
                                int* best_rows, uint8_t* desc_inout) {
    for (int i = 0; i < m; i++) {
        const int o0 = offsets[i], o1 = offsets[i + 1];
        bool bad_input = o1 < o0;
        std::vector<int> valid;
        for (int t = o0; t < o1 && !bad_input; t++) {
            if (rows[t] < -1 || rows[t] >= pool_rows) bad_input = true;
            else if (rows[t] >= 0) valid.push_back(rows[t]);
        }
        if (bad_input) {
            best_rows[i] = -2;
            continue;
        }
        if (valid.empty()) {
            best_rows[i] = -1;
            continue;
        }
        const size_t N = valid.size();
        std::vector<std::vector<int> > dist(N, std::vector<int>(N, 0));
        for (size_t a = 0; a < N; a++)
            for (size_t b = a + 1; b < N; b++) {
                const int d = hamming(pool + (size_t)valid[a] * 32, pool + (size_t)valid[b] * 32);
                dist[a][b] = d;
                dist[b][a] = d;
            }
        int best_median = INT_MAX;
        size_t best = 0;
        for (size_t a = 0; a < N; a++) {
            std::vector<int> row = dist[a];
            std::sort(row.begin(), row.end());
            const int median = row[(size_t)(0.5 * (N - 1))];
            if (median < best_median) {
                best_median = median;
                best = a;
            }
        }
        best_rows[i] = valid[best];
        if (desc_inout) std::memcpy(desc_inout + (size_t)i * 32, pool + (size_t)valid[best] * 32, 32);
    }
    return 0;
}

void orc_sincos_table(const float* x, int n, float* c, float* s) {
    for (int i = 0; i < n; i++) {
        c[i] = cosf(x[i]);
        s[i] = sinf(x[i]);
    }
}

}  // extern "C"
