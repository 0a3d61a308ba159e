// ORACLE / TEST INFRASTRUCTURE ONLY: implementation of the cv stand-in
// declared in opencv2/core/core.hpp and the imgproc / features2d / calib3d
// headers next to it.
#include "opencv2/core/core.hpp"
#include "opencv2/features2d/features2d.hpp"
#include "opencv2/imgproc/imgproc.hpp"
#include "opencv2/calib3d/calib3d.hpp"

namespace cv {

static size_t depth_size(int depth) {
    static const size_t sz[] = {1, 1, 2, 2, 4, 4, 8, 0};
    return sz[depth & 7];
}

size_t Mat::elemSize1() const { return depth_size(depth()); }

Mat::Mat(int r, int c, int type, void* d, size_t st) : Mat() {
    flags = type;
    dims = 2;
    rows = r;
    cols = c;
    data = datastart = (uchar*)d;
    step.p[1] = elemSize();
    step.p[0] = st == AUTO_STEP ? c * elemSize() : st;
    dataend = datastart + step.p[0] * r;
}

void Mat::create(int r, int c, int type) {
    if (data && rows == r && cols == c && this->type() == type) return;
    release();
    flags = type;
    dims = 2;
    rows = r;
    cols = c;
    step.p[1] = elemSize();
    step.p[0] = (size_t)c * elemSize();
    size_t bytes = step.p[0] * (size_t)r;
    buf = std::shared_ptr<uchar>(new uchar[bytes ? bytes : 1], std::default_delete<uchar[]>());
    data = datastart = buf.get();
    dataend = datastart + bytes;
}

void Mat::release() {
    buf.reset();
    data = datastart = dataend = 0;
    rows = cols = 0;
    dims = 0;
    step = MatStep();
}

Mat::Mat(const Mat& m, const Rect& roi) : Mat(m) {
    if (roi.x < 0 || roi.y < 0 || roi.x + roi.width > m.cols || roi.y + roi.height > m.rows) shim_unsupported("ROI out of range");
    data = m.data + roi.y * m.step.p[0] + roi.x * m.elemSize();
    rows = roi.height;
    cols = roi.width;
}

Mat::Mat(const Mat& m, const Range& rr, const Range& cr) : Mat(m) {
    Range r = rr.start == INT32_MIN ? Range(0, m.rows) : rr;
    Range c = cr.start == INT32_MIN ? Range(0, m.cols) : cr;
    if (r.start < 0 || r.end > m.rows || r.start > r.end || c.start < 0 || c.end > m.cols || c.start > c.end)
        shim_unsupported("row/col range out of range");
    data = m.data + r.start * m.step.p[0] + c.start * m.elemSize();
    rows = r.size();
    cols = c.size();
}

Mat Mat::clone() const {
    Mat m;
    copyTo(m);
    return m;
}

void Mat::copyTo(Mat& m) const {
    if (empty()) { m.release(); return; }
    if (m.data == data && m.step.p[0] == step.p[0] && m.rows == rows && m.cols == cols && m.type() == type()) return;
    // copy via a temporary so that overlapping source/destination is safe
    std::vector<uchar> tmp(rows * cols * elemSize());
    for (int y = 0; y < rows; y++) std::memcpy(&tmp[y * cols * elemSize()], ptr(y), cols * elemSize());
    m.create(rows, cols, type());
    for (int y = 0; y < rows; y++) std::memcpy(m.ptr(y), &tmp[y * cols * elemSize()], cols * elemSize());
}

void Mat::copyTo(const _OutputArray& m) const { copyTo(m.getMatRef()); }

static double get_elem(const Mat& m, int y, int x) {
    const uchar* p = m.ptr(y) + x * m.elemSize1();
    switch (m.depth()) {
        case CV_8U: return *(const uchar*)p;
        case CV_8S: return *(const schar*)p;
        case CV_16U: return *(const ushort*)p;
        case CV_16S: return *(const short*)p;
        case CV_32S: return *(const int*)p;
        case CV_32F: return *(const float*)p;
        case CV_64F: return *(const double*)p;
    }
    shim_unsupported("depth");
}

static void set_elem(Mat& m, int y, int x, double v) {
    uchar* p = m.ptr(y) + x * m.elemSize1();
    switch (m.depth()) {
        case CV_8U: *(uchar*)p = saturate_cast<uchar>(v); return;
        case CV_16S: *(short*)p = saturate_cast<short>(v); return;
        case CV_32S: *(int*)p = saturate_cast<int>(v); return;
        case CV_32F: *(float*)p = (float)v; return;
        case CV_64F: *(double*)p = v; return;
    }
    shim_unsupported("depth");
}

void Mat::convertTo(Mat& dst, int rtype, double alpha, double beta) const {
    if (rtype < 0) rtype = type();
    rtype = CV_MAKETYPE(CV_MAT_DEPTH(rtype), channels());
    Mat src = *this;  // keeps the source buffer alive if dst aliases it
    Mat out(rows, cols, rtype);
    const int w = cols * channels();
    for (int y = 0; y < rows; y++)
        for (int x = 0; x < w; x++) {
            double v = get_elem(src, y, x);
            if (alpha != 1 || beta != 0) {
                if (src.depth() == CV_32F || src.depth() <= CV_32S) v = (float)((float)v * (float)alpha + (float)beta);
                else v = v * alpha + beta;
            }
            set_elem(out, y, x, v);
        }
    dst = out;
}

void Mat::convertTo(const _OutputArray& dst, int rtype, double alpha, double beta) const {
    convertTo(dst.getMatRef(), rtype, alpha, beta);
}

Mat& Mat::operator=(const MatExpr& e) {
    const Mat& src = e;
    if (src.empty()) { release(); return *this; }
    if (data && rows == src.rows && cols == src.cols && type() == src.type()) {
        if (data != src.data)
            for (int y = 0; y < rows; y++) std::memcpy(ptr(y), src.ptr(y), cols * elemSize());
        return *this;
    }
    Mat::operator=(static_cast<const Mat&>(src));
    return *this;
}

Mat& Mat::operator=(const Scalar& s) {
    const int cn = channels();
    for (int y = 0; y < rows; y++)
        for (int x = 0; x < cols; x++)
            for (int c = 0; c < cn; c++) set_elem(*this, y, x * cn + c, s.val[c < 4 ? c : 0]);
    return *this;
}

MatExpr Mat::zeros(int r, int c, int type) { Mat m(r, c, type, Scalar(0)); return MatExpr(m); }
MatExpr Mat::zeros(Size sz, int type) { return zeros(sz.height, sz.width, type); }
MatExpr Mat::ones(int r, int c, int type) { Mat m(r, c, type, Scalar(1)); return MatExpr(m); }
MatExpr Mat::ones(Size sz, int type) { return ones(sz.height, sz.width, type); }
MatExpr Mat::eye(int r, int c, int type) {
    Mat m(r, c, type, Scalar(0));
    for (int i = 0; i < std::min(r, c); i++) set_elem(m, i, i, 1);
    return MatExpr(m);
}
MatExpr Mat::eye(Size sz, int type) { return eye(sz.height, sz.width, type); }

MatExpr Mat::t() const {
    Mat m(cols, rows, type());
    for (int y = 0; y < rows; y++)
        for (int x = 0; x < cols; x++) set_elem(m, x, y, get_elem(*this, y, x));
    return MatExpr(m);
}

MatExpr Mat::inv(int) const {
    if (rows != cols) shim_unsupported("inv of non-square");
    const int n = rows;
    std::vector<double> a(n * n), b(n * n, 0.0);
    for (int i = 0; i < n; i++) {
        for (int j = 0; j < n; j++) a[i * n + j] = get_elem(*this, i, j);
        b[i * n + i] = 1;
    }
    for (int c = 0; c < n; c++) {
        int p = c;
        for (int r = c + 1; r < n; r++)
            if (std::fabs(a[r * n + c]) > std::fabs(a[p * n + c])) p = r;
        for (int j = 0; j < n; j++) { std::swap(a[c * n + j], a[p * n + j]); std::swap(b[c * n + j], b[p * n + j]); }
        double d = a[c * n + c];
        for (int j = 0; j < n; j++) { a[c * n + j] /= d; b[c * n + j] /= d; }
        for (int r = 0; r < n; r++)
            if (r != c) {
                double f = a[r * n + c];
                for (int j = 0; j < n; j++) { a[r * n + j] -= f * a[c * n + j]; b[r * n + j] -= f * b[c * n + j]; }
            }
    }
    Mat m(n, n, type());
    for (int i = 0; i < n; i++)
        for (int j = 0; j < n; j++) set_elem(m, i, j, b[i * n + j]);
    return MatExpr(m);
}

double Mat::dot(const Mat& m) const {
    double s = 0;
    for (int y = 0; y < rows; y++)
        for (int x = 0; x < cols * channels(); x++) s += get_elem(*this, y, x) * get_elem(m, y, x);
    return s;
}

Mat Mat::cross(const Mat& m) const {
    Mat r(rows, cols, type());
    double a[3] = {at<float>(0), at<float>(1), at<float>(2)};
    double b[3] = {m.at<float>(0), m.at<float>(1), m.at<float>(2)};
    if (type() != CV_32F) shim_unsupported("cross");
    r.at<float>(0) = (float)(a[1] * b[2] - a[2] * b[1]);
    r.at<float>(1) = (float)(a[2] * b[0] - a[0] * b[2]);
    r.at<float>(2) = (float)(a[0] * b[1] - a[1] * b[0]);
    return r;
}

Mat Mat::reshape(int cn, int r) const {
    // OpenCV's rule: the row count stays unless given; the row width in
    // scalars (cols x channels) is redistributed over the new channel count
    Mat m = isContinuous() ? *this : clone();
    const int total_elems = m.rows * m.cols * m.channels();
    const int ncn = cn == 0 ? m.channels() : cn;
    const int nrows = r == 0 ? m.rows : r;
    if (nrows <= 0 || total_elems % nrows != 0 || (total_elems / nrows) % ncn != 0)
        shim_unsupported("reshape to a shape that does not divide the element count");
    const int ncols = total_elems / nrows / ncn;
    m.flags = CV_MAKETYPE(m.depth(), ncn);
    m.rows = nrows;
    m.cols = ncols;
    m.step.p[1] = m.elemSize();
    m.step.p[0] = (size_t)ncols * m.elemSize();
    return m;
}

void Mat::push_back(const Mat& m) {
    if (empty()) { *this = m.clone(); return; }
    Mat out(rows + m.rows, cols, type());
    for (int y = 0; y < rows; y++) std::memcpy(out.ptr(y), ptr(y), cols * elemSize());
    for (int y = 0; y < m.rows; y++) std::memcpy(out.ptr(rows + y), m.ptr(y), cols * elemSize());
    *this = out;
}

static MatExpr elementwise(const Mat& a, const Mat& b, int op) {
    if (a.rows != b.rows || a.cols != b.cols || a.type() != b.type()) shim_unsupported("elementwise size/type mismatch");
    Mat m(a.rows, a.cols, a.type());
    const int w = a.cols * a.channels();
    for (int y = 0; y < a.rows; y++)
        for (int x = 0; x < w; x++) {
            double u = get_elem(a, y, x), v = get_elem(b, y, x);
            double r;
            if (a.depth() == CV_32F) r = op == 0 ? (double)((float)u + (float)v) : (double)((float)u - (float)v);
            else r = op == 0 ? u + v : u - v;
            set_elem(m, y, x, r);
        }
    return MatExpr(m);
}

static MatExpr scaled(const Mat& a, double s) {
    Mat m(a.rows, a.cols, a.type());
    const int w = a.cols * a.channels();
    for (int y = 0; y < a.rows; y++)
        for (int x = 0; x < w; x++) {
            double u = get_elem(a, y, x);
            set_elem(m, y, x, a.depth() == CV_32F ? (double)((float)u * (float)s) : u * s);
        }
    return MatExpr(m);
}

MatExpr operator+(const Mat& a, const Mat& b) { return elementwise(a, b, 0); }
MatExpr operator-(const Mat& a, const Mat& b) { return elementwise(a, b, 1); }
MatExpr operator-(const Mat& a) { return scaled(a, -1); }
MatExpr operator*(const Mat& a, double s) { return scaled(a, s); }
MatExpr operator*(double s, const Mat& a) { return scaled(a, s); }
MatExpr operator/(const Mat& a, double s) {
    Mat m(a.rows, a.cols, a.type());
    for (int y = 0; y < a.rows; y++)
        for (int x = 0; x < a.cols * a.channels(); x++) {
            double u = get_elem(a, y, x);
            set_elem(m, y, x, a.depth() == CV_32F ? (double)((float)u / (float)s) : u / s);
        }
    return MatExpr(m);
}
MatExpr operator/(double s, const Mat& a) {
    Mat m(a.rows, a.cols, a.type());
    for (int y = 0; y < a.rows; y++)
        for (int x = 0; x < a.cols * a.channels(); x++) set_elem(m, y, x, s / get_elem(a, y, x));
    return MatExpr(m);
}

// Matrix product; like OpenCV's gemm for float inputs it accumulates in double.
MatExpr operator*(const Mat& a, const Mat& b) {
    if (a.cols != b.rows || a.type() != b.type()) shim_unsupported("gemm size/type mismatch");
    Mat m(a.rows, b.cols, a.type());
    for (int i = 0; i < a.rows; i++)
        for (int j = 0; j < b.cols; j++) {
            double s = 0;
            for (int k = 0; k < a.cols; k++) s += get_elem(a, i, k) * get_elem(b, k, j);
            set_elem(m, i, j, s);
        }
    return MatExpr(m);
}

Mat& operator+=(Mat& a, const Mat& b) { a = elementwise(a, b, 0); return a; }
Mat& operator-=(Mat& a, const Mat& b) { a = elementwise(a, b, 1); return a; }
Mat& operator*=(Mat& a, double s) { a = scaled(a, s); return a; }
Mat& operator/=(Mat& a, double s) { a = a / s; return a; }

double norm(const Mat& a, int normType) {
    double s = 0;
    for (int y = 0; y < a.rows; y++)
        for (int x = 0; x < a.cols * a.channels(); x++) {
            double v = get_elem(a, y, x);
            if (normType == NORM_L1) s += std::fabs(v);
            else if (normType == NORM_INF) s = std::max(s, std::fabs(v));
            else s += v * v;
        }
    return normType == NORM_L2 ? std::sqrt(s) : s;
}

double norm(const Mat& a, const Mat& b, int normType) {
    if (a.rows != b.rows || a.cols != b.cols || a.type() != b.type()) shim_unsupported("norm size mismatch");
    double s = 0;
    for (int y = 0; y < a.rows; y++)
        for (int x = 0; x < a.cols * a.channels(); x++) {
            double v = get_elem(a, y, x) - get_elem(b, y, x);
            if (a.depth() == CV_32F) v = (double)((float)get_elem(a, y, x) - (float)get_elem(b, y, x));
            if (normType == NORM_L1) s += std::fabs(v);
            else if (normType == NORM_INF) s = std::max(s, std::fabs(v));
            else s += v * v;
        }
    return normType == NORM_L2 ? std::sqrt(s) : s;
}

void swap(Mat& a, Mat& b) { std::swap(a, b); }
void transpose(InputArray src, OutputArray dst) { Mat t = src.getMat().t(); dst.getMatRef() = Mat(t); }

// ---------------------------------------------------------------- imgproc
void resize(InputArray _src, OutputArray _dst, Size dsize, double fx, double fy, int interpolation) {
    Mat src = _src.getMat();
    if (interpolation != INTER_LINEAR || src.type() != CV_8UC1) shim_unsupported("resize mode");
    if (dsize.width == 0 || dsize.height == 0) shim_unsupported("resize with scale factors");
    (void)fx;
    (void)fy;
    Mat tmp(dsize, CV_8UC1);
    shim_resize_linear_u8(src.data, src.step, src.cols, src.rows, tmp.data, tmp.step, dsize.width, dsize.height);
    Mat& dst = _dst.getMatRef();
    dst.create(dsize, CV_8UC1);
    for (int y = 0; y < dsize.height; y++) std::memcpy(dst.ptr(y), tmp.ptr(y), dsize.width);
}

void GaussianBlur(InputArray _src, OutputArray _dst, Size ksize, double sigmaX, double sigmaY, int borderType) {
    Mat src = _src.getMat();
    if (ksize.width != 7 || ksize.height != 7 || sigmaX != 2 || sigmaY != 2 ||
        (borderType & ~BORDER_ISOLATED) != BORDER_REFLECT_101 || src.type() != CV_8UC1)
        shim_unsupported("GaussianBlur variant");
    Mat tmp(src.rows, src.cols, CV_8UC1);
    shim_gauss7_u8(src.data, src.step, src.cols, src.rows, tmp.data, tmp.step);
    Mat& dst = _dst.getMatRef();
    dst.create(src.rows, src.cols, CV_8UC1);
    for (int y = 0; y < src.rows; y++) std::memcpy(dst.ptr(y), tmp.ptr(y), src.cols);
}

void copyMakeBorder(InputArray _src, OutputArray _dst, int top, int bottom, int left, int right, int borderType,
                    const Scalar& value) {
    (void)value;
    Mat src = _src.getMat().clone();  // source may lie inside the destination
    int bt = borderType & ~BORDER_ISOLATED;
    if (bt != BORDER_REFLECT_101 || src.type() != CV_8UC1) shim_unsupported("copyMakeBorder variant");
    Mat& dst = _dst.getMatRef();
    dst.create(src.rows + top + bottom, src.cols + left + right, CV_8UC1);
    for (int y = 0; y < dst.rows; y++) {
        int sy = shim_border_reflect101(y - top, src.rows);
        for (int x = 0; x < dst.cols; x++) dst.at<uchar>(y, x) = src.at<uchar>(sy, shim_border_reflect101(x - left, src.cols));
    }
}

// ---------------------------------------------------------------- features2d
void FAST(InputArray _img, std::vector<KeyPoint>& keypoints, int threshold, bool nonmaxSuppression) {
    Mat img = _img.getMat();
    if (!nonmaxSuppression || img.type() != CV_8UC1) shim_unsupported("FAST variant");
    keypoints.clear();
    std::vector<shim_corner> c((size_t)img.rows * img.cols / 4 + 16);
    int n = shim_fast9_u8(img.data, img.step, img.cols, img.rows, threshold, c.data(), (int)c.size());
    if (n > (int)c.size()) shim_unsupported("FAST capacity");
    for (int i = 0; i < n; i++) keypoints.push_back(KeyPoint((float)c[i].x, (float)c[i].y, 7.f, -1, (float)c[i].score));
}

void KeyPointsFilter::retainBest(std::vector<KeyPoint>&, int) { shim_unsupported("retainBest"); }

// ---------------------------------------------------------------- calib3d
// cv::undistortPoints as OpenCV 3.2's cvUndistortPoints computes it, for the
// forms ORB-SLAM2 uses (2-channel float points, a 3x3 camera matrix, 4/5/8
// distortion coefficients k1 k2 p1 p2 [k3 [k4 k5 k6]], no R, P = a 3x3
// matrix or none).  Everything in double: normalise with 1/fx, 1/fy; with
// coefficients, 5 fixed-point rounds x = (x0 - delta_x) * icdist; then
// P * R applied (R the identity) and the result rounded to float.  The
// thin-prism and tilt terms of later versions are zero for these
// coefficient counts and leave every value unchanged.
void undistortPoints(InputArray src_, OutputArray dst_, InputArray K_, InputArray dist_, InputArray R_,
                     InputArray P_) {
    const Mat src = src_.getMat();
    if (src.depth() != CV_32F || src.channels() != 2 || !src.isContinuous())
        shim_unsupported("undistortPoints: only continuous 2-channel float points");
    if (!R_.empty()) shim_unsupported("undistortPoints: R");
    const Mat K = K_.getMat();
    double A[3][3];
    for (int i = 0; i < 3; i++)
        for (int j = 0; j < 3; j++) A[i][j] = get_elem(K, i, j);
    double k[8] = {0, 0, 0, 0, 0, 0, 0, 0};
    int iters = 1;
    if (!dist_.empty()) {
        const Mat D = dist_.getMat();
        const int nk = D.rows * D.cols * D.channels();
        if (nk != 4 && nk != 5 && nk != 8) shim_unsupported("undistortPoints: distortion coefficient count");
        for (int i = 0; i < nk; i++) k[i] = get_elem(D, D.cols == 1 ? i : 0, D.cols == 1 ? 0 : i);
        iters = 5;
    }
    double RR[3][3] = {{1, 0, 0}, {0, 1, 0}, {0, 0, 1}};
    if (!P_.empty()) {
        const Mat P = P_.getMat();
        double PP[3][3];
        for (int i = 0; i < 3; i++)
            for (int j = 0; j < 3; j++) PP[i][j] = get_elem(P, i, j);
        double T[3][3];
        for (int i = 0; i < 3; i++)
            for (int j = 0; j < 3; j++) {
                double s = 0;
                for (int q = 0; q < 3; q++) s += PP[i][q] * RR[q][j];
                T[i][j] = s;
            }
        std::memcpy(RR, T, sizeof(T));
    }
    const double fx = A[0][0], fy = A[1][1], ifx = 1. / fx, ify = 1. / fy, cx = A[0][2], cy = A[1][2];
    const int n = src.rows * src.cols;
    std::vector<float> out((size_t)n * 2);
    const float* in = (const float*)src.data;
    for (int i = 0; i < n; i++) {
        double x = in[2 * i], y = in[2 * i + 1];
        double x0 = x = (x - cx) * ifx;
        double y0 = y = (y - cy) * ify;
        for (int j = 0; j < iters; j++) {
            const double r2 = x * x + y * y;
            const double icdist = (1 + ((k[7] * r2 + k[6]) * r2 + k[5]) * r2) / (1 + ((k[4] * r2 + k[1]) * r2 + k[0]) * r2);
            const double deltaX = 2 * k[2] * x * y + k[3] * (r2 + 2 * x * x);
            const double deltaY = k[2] * (r2 + 2 * y * y) + 2 * k[3] * x * y;
            x = (x0 - deltaX) * icdist;
            y = (y0 - deltaY) * icdist;
        }
        const double xx = RR[0][0] * x + RR[0][1] * y + RR[0][2];
        const double yy = RR[1][0] * x + RR[1][1] * y + RR[1][2];
        const double ww = 1. / (RR[2][0] * x + RR[2][1] * y + RR[2][2]);
        out[2 * i] = (float)(xx * ww);
        out[2 * i + 1] = (float)(yy * ww);
    }
    Mat& dst = dst_.getMatRef();
    if (dst.data != src.data || dst.type() != src.type()) dst.create(src.rows, src.cols, src.type());
    std::memcpy(dst.data, out.data(), out.size() * sizeof(float));
}

}  // namespace cv
