// Tree order and coincident-point hash of the donor search (see adt.hpp).
// Host code, compiled without floating-point contraction so that every
// product and sum is rounded as in the reference's compiled code.  Large
// subtrees and octree branches are built on worker threads: each subtree's
// node numbers follow from its size alone (a subtree of k elements takes the
// k consecutive preorder numbers after its parent's), so no counter is shared.
#include "adt.hpp"

#include <cmath>
#include <exception>
#include <mutex>
#include <system_error>
#include <thread>
#include <vector>

namespace cfdgb {
namespace adt {
namespace {

constexpr double kBig = 1.0e15;   // BIGVALUE, UniTioga/codetypes.h:52
constexpr double kTol = 1.0e-10;  // TOL, UniTioga/codetypes.h:54
constexpr int kParallelSize = 1 << 16;
constexpr int kParallelDepth = 4;

// Subtree tasks: each runs on a thread of its own when one can be started,
// else in the caller; an exception thrown in a thread (an allocation that
// failed) is kept and rethrown by join(), and every thread is joined before
// the object goes away.
class Tasks {
  public:
    template <class F>
    void run(bool parallel, F f) {
        if (parallel) {
            try {
                ts_.emplace_back([this, f]() {
                    try {
                        f();
                    } catch (...) {
                        std::lock_guard<std::mutex> g(mu_);
                        if (!err_) err_ = std::current_exception();
                    }
                });
                return;
            } catch (const std::system_error&) {
                // no thread to be had: run it here
            }
        }
        f();
    }
    void join() {
        for (auto& t : ts_) t.join();
        ts_.clear();
        if (err_) std::rethrow_exception(err_);
    }
    ~Tasks() {
        for (auto& t : ts_)
            if (t.joinable()) t.join();
    }

  private:
    std::vector<std::thread> ts_;
    std::exception_ptr err_;
    std::mutex mu_;
};

// One Jacobi sweep set of kaiser() on a symmetric 2x2 matrix held by columns,
// then the columns scaled to unit length (zero columns stay zero).
void kaiser2(double a[2][2]) {
    double ss = 0;
    for (int i = 0; i < 2; i++)
        for (int j = 0; j < 2; j++) ss += a[i][j] * a[i][j];
    const double eps = 1.0e-12 * ss / 2;
    for (int sweep = 0; sweep < 100; sweep++) {
        // the only off-diagonal pair of a 2x2 matrix: columns 0 and 1
        double half_p = 0, q = 0;
        for (int k = 0; k < 2; k++) {
            half_p += a[k][0] * a[k][1];
            q += (a[k][0] + a[k][1]) * (a[k][0] - a[k][1]);
        }
        const double p = 2 * half_p;
        const double ap = std::fabs(p);
        if (ap < eps && q >= 0) break;  // every pair skipped: converged
        const double aq = std::fabs(q);
        double c2, s2;  // cos and sin of twice the angle
        if (ap <= aq) {
            const double t = ap / aq;
            c2 = 1 / std::sqrt(1 + t * t);
            s2 = t * c2;
        } else {
            const double t = aq / ap;
            s2 = 1 / std::sqrt(1 + t * t);
            c2 = s2 * t;
        }
        double c = std::sqrt((1 + c2) / 2);
        double s = s2 / (2 * c);
        if (q < 0) {
            const double t = c;
            c = s;
            s = t;
        }
        if (p < 0) s = -s;
        for (int k = 0; k < 2; k++) {
            const double a0 = a[k][0];
            a[k][0] = a0 * c + a[k][1] * s;
            a[k][1] = -a0 * s + a[k][1] * c;
        }
    }
    double len[2];
    for (int i = 0; i < 2; i++) {
        double t = 0;
        for (int j = 0; j < 2; j++) t += a[j][i] * a[j][i];
        len[i] = std::sqrt(t);
    }
    for (int i = 0; i < 2; i++)
        for (int j = 0; j < 2; j++) a[j][i] = len[i] > 0 ? a[j][i] / len[i] : 0.0;
}

// A tree element: its box and its number.  The median split reorders whole
// elements, so each level reads its cut coordinate sequentially; the
// reference reorders an index array and a gathered coordinate array in the
// same way, so the order of every comparison and exchange is the same.
struct Elem {
    double c[4];  // min x, min y, max x, max y
    int id;
};

inline void swap_at(Elem* e, int a, int b) {
    const Elem t = e[a];
    e[a] = e[b];
    e[b] = t;
}

// median.cpp's find_median: one Hoare pass about the middle entry clamped to
// the two ends' range, then a recursion into the side that still holds the
// median position.  ilow / ihigh are in-out, as the reference's references.
void partial_median(Elem* e, int cut, int n, int& ilow, int& ihigh) {
    int low = ilow, high = ihigh;
    const int mid = (low + high) / 2;
    const int half = (n - 1) / 2, half1 = half + 1;
    double lo = e[low].c[cut], hi = e[high].c[cut], pivot = e[mid].c[cut];
    if (lo > hi) {
        const double t = lo;
        lo = hi;
        hi = t;
    }
    if (pivot > hi) pivot = hi;
    else if (pivot < lo) pivot = lo;
    int i = low, j = high;
    bool again = true;
    while (again) {
        again = false;
        while (!(e[i].c[cut] >= pivot)) ++i;
        while (!(e[j].c[cut] <= pivot)) --j;
        if (i < j) {
            swap_at(e, i, j);
            ++i;
            --j;
            again = i <= j;
        }
    }
    if (n % 2 == 0) {
        if (j == half && i == half1) {
            // split exactly in two: the largest of the left part goes to the middle
            int at = j;
            for (int k = 0; k < half; k++)
                if (e[k].c[cut] > e[at].c[cut]) at = k;
            if (at != j) swap_at(e, at, j);
            return;
        }
        if (j < half) low = i;
        if (i > half1) high = j;
        if (i != j) {
            if (low < high - 1) partial_median(e, cut, n, low, high);
            return;
        }
        if (i == half) low = half;
        if (j == half1) high = half1;
    } else {
        if (j < half) low = i;
        if (i > half) high = j;
        if (i != j) {
            if (low < high - 1) partial_median(e, cut, n, low, high);
            ilow = low;
            ihigh = high;
            return;
        }
        if (i == half) {
            ilow = low;
            ihigh = high;
            return;
        }
    }
    if (low < high - 1) {
        ilow = low;
        ihigh = high;
        partial_median(e, cut, n, low, high);
    }
}

// find_median_wrap: the element at (n+1)/2 - 1 is the split element afterwards.
void median_split(Elem* e, int cut, int n) {
    if (n <= 2) {
        if (n == 2 && e[0].c[cut] > e[1].c[cut]) swap_at(e, 0, 1);
        return;
    }
    int ilow = 0, ihigh = n - 1;
    const int half = (n - 1) / 2;
    partial_median(e, cut, n, ilow, ihigh);
    if (n % 2 == 0) {
        if (e[half].c[cut] > e[half + 1].c[cut]) swap_at(e, half, half + 1);
    } else if (e[ilow].c[cut] > e[ihigh].c[cut]) {
        swap_at(e, ilow, ihigh);
    }
}

// buildADTrecursion with explicit node numbers: the subtree of `nav` elements
// rooted at node `base` holds nodes base .. base+nav-1; its split element
// takes `base`, the left part base+1 .., the right part base+nleft ..
void build(int* node, Elem* e, int nav, int level, int base, int depth) {
    while (nav > 1) {
        median_split(e, level % 4, nav);
        const int nleft = (nav + 1) / 2;
        node[e[nleft - 1].id] = base;
        if (nleft > 1) {
            if (nav >= kParallelSize && depth < kParallelDepth) {
                Tasks tasks;
                tasks.run(true, [=] { build(node, e, nleft - 1, level + 1, base + 1, depth + 1); });
                build(node, e + nleft, nav - nleft, level + 1, base + nleft, depth + 1);
                tasks.join();
                return;
            }
            build(node, e, nleft - 1, level + 1, base + 1, depth + 1);
        }
        // the right part, iteratively
        e += nleft;
        nav -= nleft;
        level += 1;
        base += nleft;
        depth += 1;
    }
    if (nav == 1) node[e[0].id] = base;
}

// uniqNodesTree: split at the box centre into four quadrants while more than
// 20 points remain and they do not all fall in one; compare pairs in a leaf.
void octree(const double* x, const int* tag, double* res, int* xtag, int* avail, int nav, int depth) {
    bool leaf = true;
    if (nav > 20) {
        double mn[2] = {kBig, kBig}, mx[2] = {-kBig, -kBig};
        for (int i = 0; i < nav; i++)
            for (int j = 0; j < 2; j++) {
                const double v = x[2 * (size_t)avail[i] + j];
                mn[j] = mn[j] < v ? mn[j] : v;
                mx[j] = mx[j] > v ? mx[j] : v;
            }
        double mid[2], half[2];
        for (int j = 0; j < 2; j++) {
            mid[j] = (mx[j] + mn[j]) * 0.5;
            half[j] = (mx[j] - mn[j]) * 0.5 + kTol;
        }
        auto quadrant = [&](int p) {
            const int ix = (int)(std::floor((x[2 * (size_t)p] - mid[0]) / half[0]) + 1);
            const int iy = (int)(std::floor((x[2 * (size_t)p + 1] - mid[1]) / half[1]) + 1);
            return 2 * ix + iy;
        };
        int cnt[4] = {0, 0, 0, 0};
        std::vector<int> q(nav);
        bool bad = false;  // a quadrant outside 0..3 (coordinates so large that TOL is below their spacing)
        for (int i = 0; i < nav; i++) {
            q[i] = quadrant(avail[i]);
            if (q[i] < 0 || q[i] > 3) bad = true;
            else cnt[q[i]]++;
        }
        leaf = bad;
        for (int j = 0; j < 4; j++)
            if (cnt[j] == nav) leaf = true;
        if (!leaf) {
            int start[5] = {0, 0, 0, 0, 0};
            for (int j = 0; j < 4; j++) start[j + 1] = start[j] + cnt[j];
            std::vector<int> tmp(nav);
            for (int i = 0; i < nav; i++) tmp[start[q[i]] + --cnt[q[i]]] = avail[i];  // each quadrant filled from its end
            for (int i = 0; i < nav; i++) avail[i] = tmp[i];
            Tasks tasks;
            for (int j = 0; j < 4; j++) {
                const int len = start[j + 1] - start[j];
                if (len <= 0) continue;
                int* sub = avail + start[j];
                tasks.run(nav >= kParallelSize && depth < kParallelDepth,
                          [=] { octree(x, tag, res, xtag, sub, len, depth + 1); });
            }
            tasks.join();
        }
    }
    if (!leaf) return;
    for (int i = 0; i < nav; i++) {
        const int p1 = avail[i];
        for (int j = i + 1; j < nav; j++) {
            const int p2 = avail[j];
            if (std::fabs(x[2 * (size_t)p1] - x[2 * (size_t)p2]) + std::fabs(x[2 * (size_t)p1 + 1] - x[2 * (size_t)p2 + 1]) <
                    kTol &&
                tag[p1] == tag[p2]) {
                const int lo = p1 < p2 ? p1 : p2, hi = p1 < p2 ? p2 : p1;
                res[lo] = res[p1] > res[p2] ? res[p1] : res[p2];
                xtag[hi] = xtag[lo];
            }
        }
    }
}

}  // namespace

Obb find_obb(const double* xy, long long n) {
    Obb o{};
    for (long long i = 0; i < n; i++)
        for (int j = 0; j < 2; j++) o.xc[j] += xy[2 * i + j];
    for (int j = 0; j < 2; j++) o.xc[j] = o.xc[j] / n;
    if (n <= 2) {
        o.vec[0][0] = o.vec[1][1] = 1;
        for (int j = 0; j < 2; j++) {
            if (n == 1) {
                o.dxc[j] = 1e-3;
            } else {
                // the reference's max macro binds the halving to its second operand only
                const double d = std::fabs(xy[2 + j] - xy[j]);
                o.dxc[j] = 1e-3 > d ? 1e-3 : d * 0.5;
            }
        }
        return o;
    }
    double a[2][2] = {{0, 0}, {0, 0}};
    for (long long i = 0; i < n; i++)
        for (int j = 0; j < 2; j++)
            for (int k = j; k < 2; k++) a[j][k] += (xy[2 * i + j] - o.xc[j]) * (xy[2 * i + k] - o.xc[k]);
    a[1][0] = a[0][1];
    kaiser2(a);
    double mn[2] = {kBig, kBig}, mx[2] = {-kBig, -kBig};
    for (int j = 0; j < 2; j++)
        for (int k = 0; k < 2; k++) o.vec[j][k] = a[j][k];
    for (long long i = 0; i < n; i++)
        for (int j = 0; j < 2; j++) {
            double d = 0;
            for (int k = 0; k < 2; k++) d += (xy[2 * i + k] - o.xc[k]) * o.vec[j][k];
            mx[j] = mx[j] > d ? mx[j] : d;
            mn[j] = mn[j] < d ? mn[j] : d;
        }
    double ctr[2];
    for (int j = 0; j < 2; j++) {
        o.dxc[j] = (mx[j] - mn[j]) * 0.5 * 1.01;
        ctr[j] = (mx[j] + mn[j]) * 0.5;
    }
    for (int j = 0; j < 2; j++)
        for (int k = 0; k < 2; k++) o.xc[j] += ctr[k] * o.vec[k][j];
    return o;
}

std::vector<int> node_order(int nelem, const double* box) {
    std::vector<int> node(nelem > 0 ? nelem : 0, -1);
    std::vector<Elem> e(nelem > 0 ? nelem : 0);
    for (int i = 0; i < nelem; i++) {
        for (int k = 0; k < 4; k++) e[i].c[k] = box[4 * (size_t)i + k];
        e[i].id = i;
    }
    if (nelem > 0) build(node.data(), e.data(), nelem, 0, 0, 0);
    return node;
}

std::vector<int> tree_ranks(int ncell, const double* xy, const int* cv, const int* order, const unsigned char* cross) {
    std::vector<int> elem_cell;
    std::vector<double> box;
    for (int p = ncell - 1; p >= 0; p--) {
        const int c = order[p];
        if (!cross[c]) continue;
        const int nv = cv[4 * (size_t)c + 3] < 0 ? 3 : 4;
        double mn[2] = {kBig, kBig}, mx[2] = {-kBig, -kBig};
        for (int m = 0; m < nv; m++)
            for (int j = 0; j < 2; j++) {
                const double x = xy[2 * (size_t)cv[4 * (size_t)c + m] + j];
                mn[j] = mn[j] < x ? mn[j] : x;
                mx[j] = mx[j] > x ? mx[j] : x;
            }
        elem_cell.push_back(c);
        box.insert(box.end(), {mn[0], mn[1], mx[0], mx[1]});
    }
    const std::vector<int> node = node_order((int)elem_cell.size(), box.data());
    std::vector<int> rank(ncell, -1);
    for (size_t l = 0; l < elem_cell.size(); l++) rank[elem_cell[l]] = node[l];
    return rank;
}

void coincident(long long n, const double* xy, const int* tag, double* res, int* xtag) {
    std::vector<int> avail(n);
    for (long long i = 0; i < n; i++) avail[i] = (int)i, xtag[i] = (int)i;
    if (n > 0) octree(xy, tag, res, xtag, avail.data(), (int)n, 0);
}

}  // namespace adt
}  // namespace cfdgb
