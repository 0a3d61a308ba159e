// ORACLE / TEST INFRASTRUCTURE ONLY.
// A minimal stand-in for the parts of the OpenCV 2.x/3.x core API that
// ORB-SLAM2's src/ORBextractor.cc, src/ORBmatcher.cc and src/Frame.cc (and the
// headers they include) use, so that those files compile unmodified for use as
// the parity oracle.  Only the behaviour those files rely on is implemented;
// everything else is declared so the headers parse, and aborts if called.
#ifndef CVSHIM_CORE_HPP
#define CVSHIM_CORE_HPP

#include <algorithm>
#include <cassert>
#include <cmath>
#include <climits>
#include <cstdint>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <iostream>
#include <map>
#include <memory>
#include <sstream>
#include <fstream>
#include <limits>
#include <list>
#include <string>
#include <vector>

#include "../../cvshim_prims.h"

#define CV_PI 3.1415926535897932384626433832795
#define CV_8U 0
#define CV_8S 1
#define CV_16U 2
#define CV_16S 3
#define CV_32S 4
#define CV_32F 5
#define CV_64F 6
#define CV_CN_SHIFT 3
#define CV_MAT_DEPTH(t) ((t) & 7)
#define CV_MAT_CN(t) ((((t) >> CV_CN_SHIFT) & 511) + 1)
#define CV_MAKETYPE(d, cn) (CV_MAT_DEPTH(d) + (((cn)-1) << CV_CN_SHIFT))
#define CV_8UC1 CV_MAKETYPE(CV_8U, 1)
#define CV_8UC2 CV_MAKETYPE(CV_8U, 2)
#define CV_8UC3 CV_MAKETYPE(CV_8U, 3)
#define CV_32FC1 CV_MAKETYPE(CV_32F, 1)
#define CV_32FC2 CV_MAKETYPE(CV_32F, 2)
#define CV_32SC1 CV_MAKETYPE(CV_32S, 1)
#define CV_64FC1 CV_MAKETYPE(CV_64F, 1)

namespace cv {

typedef unsigned char uchar;
typedef signed char schar;
typedef unsigned short ushort;

[[noreturn]] inline void shim_unsupported(const char* what) {
    std::fprintf(stderr, "cvshim: unsupported call: %s\n", what);
    std::abort();
}

inline int cvRound(double v) { return shim_cvround_d(v); }
inline int cvRound(float v) { return shim_cvround_f(v); }
inline int cvRound(int v) { return v; }
inline int cvFloor(double v) { int i = (int)v; return i - (i > v); }
inline int cvFloor(float v) { int i = (int)v; return i - (i > v); }
inline int cvCeil(double v) { int i = (int)v; return i + (i < v); }
inline int cvCeil(float v) { int i = (int)v; return i + (i < v); }

template <typename T> inline T saturate_cast(double v);
template <> inline uchar saturate_cast<uchar>(double v) { int i = cvRound(v); return (uchar)(i < 0 ? 0 : (i > 255 ? 255 : i)); }
template <> inline short saturate_cast<short>(double v) { int i = cvRound(v); return (short)(i < -32768 ? -32768 : (i > 32767 ? 32767 : i)); }
template <> inline int saturate_cast<int>(double v) { return cvRound(v); }
template <> inline float saturate_cast<float>(double v) { return (float)v; }
template <> inline double saturate_cast<double>(double v) { return v; }

inline float fastAtan2(float y, float x) { return shim_fast_atan2(y, x); }

template <typename T> struct Point_ {
    T x, y;
    Point_() : x(0), y(0) {}
    Point_(T _x, T _y) : x(_x), y(_y) {}
    template <typename T2> operator Point_<T2>() const { return Point_<T2>(conv<T2>(x), conv<T2>(y)); }
    template <typename T2> static T2 conv(T v) { return (T2)v; }
    T dot(const Point_& p) const { return x * p.x + y * p.y; }
};
template <> template <> inline int Point_<float>::conv<int>(float v) { return cvRound(v); }
template <> template <> inline int Point_<double>::conv<int>(double v) { return cvRound(v); }
template <typename T, typename S> inline Point_<T>& operator*=(Point_<T>& a, S b) { a.x = (T)(a.x * b); a.y = (T)(a.y * b); return a; }
template <typename T> inline Point_<T>& operator+=(Point_<T>& a, const Point_<T>& b) { a.x += b.x; a.y += b.y; return a; }
template <typename T> inline Point_<T>& operator-=(Point_<T>& a, const Point_<T>& b) { a.x -= b.x; a.y -= b.y; return a; }
template <typename T> inline Point_<T> operator+(const Point_<T>& a, const Point_<T>& b) { return Point_<T>(a.x + b.x, a.y + b.y); }
template <typename T> inline Point_<T> operator-(const Point_<T>& a, const Point_<T>& b) { return Point_<T>(a.x - b.x, a.y - b.y); }
template <typename T> inline bool operator==(const Point_<T>& a, const Point_<T>& b) { return a.x == b.x && a.y == b.y; }
template <typename T> inline bool operator!=(const Point_<T>& a, const Point_<T>& b) { return !(a == b); }
typedef Point_<int> Point2i;
typedef Point_<float> Point2f;
typedef Point_<double> Point2d;
typedef Point2i Point;

template <typename T> struct Point3_ {
    T x, y, z;
    Point3_() : x(0), y(0), z(0) {}
    Point3_(T _x, T _y, T _z) : x(_x), y(_y), z(_z) {}
};
typedef Point3_<float> Point3f;
typedef Point3_<double> Point3d;

template <typename T> struct Size_ {
    T width, height;
    Size_() : width(0), height(0) {}
    Size_(T w, T h) : width(w), height(h) {}
    T area() const { return width * height; }
};
typedef Size_<int> Size;
typedef Size_<float> Size2f;

template <typename T> struct Rect_ {
    T x, y, width, height;
    Rect_() : x(0), y(0), width(0), height(0) {}
    Rect_(T _x, T _y, T w, T h) : x(_x), y(_y), width(w), height(h) {}
};
typedef Rect_<int> Rect;

struct Range {
    int start, end;
    Range() : start(0), end(0) {}
    Range(int s, int e) : start(s), end(e) {}
    static Range all() { return Range(INT32_MIN, INT32_MAX); }
    int size() const { return end - start; }
};

struct Scalar {
    double val[4];
    Scalar(double v0 = 0, double v1 = 0, double v2 = 0, double v3 = 0) { val[0] = v0; val[1] = v1; val[2] = v2; val[3] = v3; }
    double operator[](int i) const { return val[i]; }
};

class KeyPoint {
public:
    Point2f pt;
    float size;
    float angle;
    float response;
    int octave;
    int class_id;
    KeyPoint() : pt(0, 0), size(0), angle(-1), response(0), octave(0), class_id(-1) {}
    KeyPoint(Point2f _pt, float _size, float _angle = -1, float _response = 0, int _octave = 0, int _class_id = -1)
        : pt(_pt), size(_size), angle(_angle), response(_response), octave(_octave), class_id(_class_id) {}
    KeyPoint(float x, float y, float _size, float _angle = -1, float _response = 0, int _octave = 0, int _class_id = -1)
        : pt(x, y), size(_size), angle(_angle), response(_response), octave(_octave), class_id(_class_id) {}
};

class DMatch {
public:
    int queryIdx, trainIdx, imgIdx;
    float distance;
    DMatch() : queryIdx(-1), trainIdx(-1), imgIdx(-1), distance(0) {}
};

struct MatStep {
    size_t p[2];
    MatStep() { p[0] = p[1] = 0; }
    operator size_t() const { return p[0]; }
    size_t operator[](int i) const { return p[i]; }
};

class MatExpr;
class _InputArray;
class _OutputArray;

class Mat {
public:
    int flags;  // type
    int dims;
    int rows, cols;
    uchar* data;
    std::shared_ptr<uchar> buf;
    uchar* datastart;
    uchar* dataend;
    MatStep step;
    enum { AUTO_STEP = 0 };

    Mat() : flags(0), dims(0), rows(0), cols(0), data(0), datastart(0), dataend(0) {}
    Mat(int r, int c, int type) : Mat() { create(r, c, type); }
    Mat(Size sz, int type) : Mat() { create(sz.height, sz.width, type); }
    Mat(int r, int c, int type, const Scalar& s) : Mat() { create(r, c, type); *this = s; }
    Mat(Size sz, int type, const Scalar& s) : Mat() { create(sz.height, sz.width, type); *this = s; }
    Mat(int r, int c, int type, void* d, size_t st = AUTO_STEP);
    Mat(const Mat& m, const Rect& roi);
    Mat(const Mat& m, const Range& rr, const Range& cr = Range::all());
    Mat(const Mat& m) = default;
    Mat& operator=(const Mat& m) = default;
    Mat& operator=(const MatExpr& e);
    Mat& operator=(const Scalar& s);
    template <typename T> explicit Mat(const std::vector<T>& v, bool copyData = false);

    void create(int r, int c, int type);
    void create(Size sz, int type) { create(sz.height, sz.width, type); }
    void release();
    bool empty() const { return data == 0 || rows * cols == 0; }
    int type() const { return flags & 0xFFF; }
    int depth() const { return CV_MAT_DEPTH(flags); }
    int channels() const { return CV_MAT_CN(flags); }
    size_t elemSize1() const;
    size_t elemSize() const { return elemSize1() * channels(); }
    size_t step1(int i = 0) const { return step.p[i] / elemSize1(); }
    size_t total() const { return (size_t)rows * cols; }
    bool isContinuous() const { return rows <= 1 || step.p[0] == cols * elemSize(); }
    bool isSubmatrix() const { return data != datastart || (size_t)(dataend - datastart) != step.p[0] * rows; }
    Size size() const { return Size(cols, rows); }

    Mat row(int y) const { return Mat(*this, Range(y, y + 1), Range::all()); }
    Mat col(int x) const { return Mat(*this, Range::all(), Range(x, x + 1)); }
    Mat rowRange(int s, int e) const { return Mat(*this, Range(s, e), Range::all()); }
    Mat rowRange(const Range& r) const { return Mat(*this, r, Range::all()); }
    Mat colRange(int s, int e) const { return Mat(*this, Range::all(), Range(s, e)); }
    Mat colRange(const Range& r) const { return Mat(*this, Range::all(), r); }
    Mat operator()(const Rect& roi) const { return Mat(*this, roi); }
    Mat operator()(const Range& rr, const Range& cr) const { return Mat(*this, rr, cr); }

    Mat clone() const;
    void copyTo(Mat& m) const;
    void copyTo(const _OutputArray& m) const;
    void convertTo(const _OutputArray& m, int rtype, double alpha = 1, double beta = 0) const;
    void convertTo(Mat& m, int rtype, double alpha = 1, double beta = 0) const;
    MatExpr t() const;
    MatExpr inv(int method = 0) const;
    double dot(const Mat& m) const;
    Mat cross(const Mat& m) const;
    Mat reshape(int cn, int r = 0) const;
    Mat& setTo(const Scalar& s) { *this = s; return *this; }
    void push_back(const Mat& m);

    template <typename T> T& at(int r, int c) { return ((T*)(data + step.p[0] * r))[c]; }
    template <typename T> const T& at(int r, int c) const { return ((const T*)(data + step.p[0] * r))[c]; }
    template <typename T> T& at(int i) {
        if (rows == 1 || isContinuous()) return ((T*)data)[i];
        return at<T>(i, 0);
    }
    template <typename T> const T& at(int i) const {
        if (rows == 1 || isContinuous()) return ((const T*)data)[i];
        return at<T>(i, 0);
    }
    template <typename T> T& at(Point pt) { return at<T>(pt.y, pt.x); }
    template <typename T> const T& at(Point pt) const { return at<T>(pt.y, pt.x); }
    uchar* ptr(int r = 0) { return data + step.p[0] * r; }
    const uchar* ptr(int r = 0) const { return data + step.p[0] * r; }
    template <typename T> T* ptr(int r = 0) { return (T*)(data + step.p[0] * r); }
    template <typename T> const T* ptr(int r = 0) const { return (const T*)(data + step.p[0] * r); }

    static MatExpr zeros(int r, int c, int type);
    static MatExpr zeros(Size sz, int type);
    static MatExpr ones(int r, int c, int type);
    static MatExpr ones(Size sz, int type);
    static MatExpr eye(int r, int c, int type);
    static MatExpr eye(Size sz, int type);
};

// Result of a matrix expression.  Assigning it to an existing Mat of the same
// size and type writes into that Mat's buffer (OpenCV's MatExpr semantics,
// which ORB-SLAM2 relies on when it fills descriptor row ranges).
class MatExpr : public Mat {
public:
    MatExpr() {}
    explicit MatExpr(const Mat& m) : Mat(m) {}
};

template <typename T> struct DataDepth;
template <> struct DataDepth<uchar> { enum { value = CV_8U }; };
template <> struct DataDepth<int> { enum { value = CV_32S }; };
template <> struct DataDepth<float> { enum { value = CV_32F }; };
template <> struct DataDepth<double> { enum { value = CV_64F }; };

template <typename T> Mat::Mat(const std::vector<T>& v, bool copyData) : Mat() {
    create((int)v.size(), 1, DataDepth<T>::value);
    (void)copyData;
    if (!v.empty()) std::memcpy(data, v.data(), v.size() * sizeof(T));
}

template <typename T> class MatCommaInitializer_;
template <typename T> class Mat_ : public Mat {
public:
    Mat_() {}
    Mat_(int r, int c) : Mat(r, c, DataDepth<T>::value) {}
    Mat_(const Mat& m) : Mat(m) {}
    T& operator()(int r, int c) { return at<T>(r, c); }
};
template <typename T> class MatCommaInitializer_ {
public:
    Mat_<T> m;
    int idx;
    MatCommaInitializer_(const Mat_<T>& _m, T v) : m(_m), idx(0) { put(v); }
    void put(T v) { ((T*)m.data)[idx++] = v; }
    template <typename T2> MatCommaInitializer_& operator,(T2 v) { put((T)v); return *this; }
    operator Mat() const { return m; }
    operator Mat_<T>() const { return m; }
};
template <typename T, typename T2> MatCommaInitializer_<T> operator<<(const Mat_<T>& m, T2 v) { return MatCommaInitializer_<T>(m, (T)v); }

MatExpr operator+(const Mat& a, const Mat& b);
MatExpr operator-(const Mat& a, const Mat& b);
MatExpr operator-(const Mat& a);
MatExpr operator*(const Mat& a, const Mat& b);
MatExpr operator*(const Mat& a, double s);
MatExpr operator*(double s, const Mat& a);
MatExpr operator/(const Mat& a, double s);
MatExpr operator/(double s, const Mat& a);
Mat& operator+=(Mat& a, const Mat& b);
Mat& operator-=(Mat& a, const Mat& b);
Mat& operator*=(Mat& a, double s);
Mat& operator/=(Mat& a, double s);

enum { NORM_INF = 1, NORM_L1 = 2, NORM_L2 = 4, NORM_HAMMING = 6 };
double norm(const Mat& a, int normType = NORM_L2);
double norm(const Mat& a, const Mat& b, int normType = NORM_L2);

class _InputArray {
public:
    const Mat* m;
    Mat tmp;
    _InputArray() : m(0) {}
    _InputArray(const Mat& mat) : m(&mat) {}
    _InputArray(const MatExpr& e) : m(0), tmp(e) { m = &tmp; }
    template <typename T> _InputArray(const std::vector<T>& v) : m(0), tmp(v) { m = &tmp; }
    Mat getMat(int i = -1) const { (void)i; return m ? *m : Mat(); }
    bool empty() const { return m == 0 || m->empty(); }
    int type() const { return m ? m->type() : 0; }
};
typedef const _InputArray& InputArray;

class _OutputArray : public _InputArray {
public:
    Mat* om;
    _OutputArray() : om(0) {}
    _OutputArray(Mat& mat) : _InputArray(mat), om(&mat) {}
    void create(int r, int c, int type) const { om->create(r, c, type); }
    void create(Size sz, int type) const { om->create(sz.height, sz.width, type); }
    Mat getMat(int i = -1) const { (void)i; return *om; }
    Mat& getMatRef() const { return *om; }
    void release() const { om->release(); }
    bool empty() const { return om == 0 || om->empty(); }
};
typedef const _OutputArray& OutputArray;
typedef const _OutputArray& InputOutputArray;
inline const _InputArray& noArray() { static _InputArray a; return a; }

void swap(Mat& a, Mat& b);
void transpose(InputArray src, OutputArray dst);

// Persistence stubs (only parsed by DBoW2's TemplatedVocabulary, never called).
class FileNode {
public:
    FileNode operator[](const std::string&) const { shim_unsupported("FileNode"); }
    FileNode operator[](const char*) const { shim_unsupported("FileNode"); }
    FileNode operator[](int) const { shim_unsupported("FileNode"); }
    size_t size() const { shim_unsupported("FileNode"); }
    operator int() const { shim_unsupported("FileNode"); }
    operator float() const { shim_unsupported("FileNode"); }
    operator double() const { shim_unsupported("FileNode"); }
    operator std::string() const { shim_unsupported("FileNode"); }
};
class FileStorage {
public:
    enum { READ = 0, WRITE = 1 };
    FileStorage() {}
    FileStorage(const std::string&, int) { shim_unsupported("FileStorage"); }
    bool isOpened() const { return false; }
    FileNode operator[](const std::string&) const { shim_unsupported("FileStorage"); }
    FileNode operator[](const char*) const { shim_unsupported("FileStorage"); }
};
template <typename T> inline FileStorage& operator<<(FileStorage& fs, const T&) { shim_unsupported("FileStorage<<"); return fs; }

}  // namespace cv

#endif
