// Element orders of the reference's brick topologies.
//
// BrickTopology numbers the elements of a brick along the Hilbert curve
// through their centroids, even on one rank: BrickMesh.partition sorts the
// elements (created in Cartesian order, x fastest) by the Hilbert code of
// their centroid (src/Numerics/Mesh/BrickMesh.jl:531-560, 617-627), with the
// code from centroidtocode (:112-150) and hilbertcode (:40-90).
// StackedBrickTopology builds that BrickTopology over the horizontal
// directions and stacks each base element's column contiguously, the
// vertical index fastest (src/Numerics/Mesh/Topologies.jl:632-715).
//
// The library's generated bricks keep columns contiguous with the columns in
// x-then-y order.  cmdg_brick_element_order gives the permutation between
// the two, and a mesh created with the StackedBrickTopology order
// (cmdg_mesh_create_brick_ordered) runs directly on states in the
// reference's element order.
//
// hilbertcode is John Skilling's transform of axes to the transposed
// Hilbert index ("Programming the Hilbert curve", AIP Conf. Proc. 707, 2004),
// followed by the transposition of the n words into the Hilbert integer
// that the reference applies; the element codes are the centroids scaled to
// [0, 2^64 - 1] and floored exactly.
#include <algorithm>
#include <array>
#include <cmath>
#include <cstring>
#include <numeric>

#include "cmdg_internal.h"

namespace cmdg {

// Hilbert index of the n coordinates X (each `bits` bits wide) as n words,
// most significant word first (BrickMesh.jl:40-90).
void hilbert_code(const uint64_t* Y, int n, int bits, uint64_t* H) {
    uint64_t X[3];
    for (int i = 0; i < n; ++i) X[i] = Y[i];
    const uint64_t M = (uint64_t)1 << (bits - 1);
    // inverse undo: axes to the transposed index
    for (uint64_t Q = M; Q > 1; Q >>= 1) {
        const uint64_t P = Q - 1;
        for (int i = 0; i < n; ++i) {
            if (X[i] & Q) {
                X[0] ^= P;
            } else {
                const uint64_t t = (X[0] ^ X[i]) & P;
                X[0] ^= t;
                X[i] ^= t;
            }
        }
    }
    // Gray encode
    for (int i = 1; i < n; ++i) X[i] ^= X[i - 1];
    uint64_t t = 0;
    for (uint64_t Q = M; Q > 1; Q >>= 1)
        if (X[n - 1] & Q) t ^= Q - 1;
    for (int i = 0; i < n; ++i) X[i] ^= t;
    // transpose: bit k of the interleaved index is bit (k / n) of word
    // n - 1 - (k mod n); the index's bits fill H from its last word up
    for (int i = 0; i < n; ++i) H[i] = 0;
    for (int i = 0; i < n; ++i)
        for (int j = 0; j < bits; ++j) {
            const int k = i * bits + j;
            const uint64_t bit = (X[n - 1 - (k % n)] >> (k / n)) & 1u;
            H[n - 1 - i] |= bit << j;
        }
}

// floor((2^64 - 1) c) for c in [0, 1], exact: c = m 2^-s with an integer
// mantissa m < 2^53, so the product is ((m 2^64) - m) 2^-s.
static uint64_t scale_unit(double c) {
    if (!(c > 0)) return 0;
    if (c >= 1) return ~(uint64_t)0;
    int e2 = 0;
    const double f = std::frexp(c, &e2);  // c = f 2^e2, f in [0.5, 1)
    const uint64_t m = (uint64_t)std::ldexp(f, 53);
    const int s = 53 - e2;               // c = m 2^-s, s > 53
    if (s >= 117) return 0;
    const unsigned __int128 num = ((unsigned __int128)m << 64) - m;
    return (uint64_t)(num >> s);
}

// Codes of element centroids (d x nelem, element-major) as centroidtocode
// computes them on one rank (BrickMesh.jl:112-150): centroid minus the
// minimum over elements, divided by the extent (a zero extent replaced by
// the largest one, all-zero extents by one), scaled to 64 bits.
void centroid_codes(const double* centroids, int d, int64_t nelem, std::vector<uint64_t>& code) {
    std::array<double, 3> lo, hi, size;
    for (int i = 0; i < d; ++i) {
        lo[i] = INFINITY;
        hi[i] = -INFINITY;
    }
    for (int64_t e = 0; e < nelem; ++e)
        for (int i = 0; i < d; ++i) {
            lo[i] = std::min(lo[i], centroids[e * d + i]);
            hi[i] = std::max(hi[i], centroids[e * d + i]);
        }
    double biggest = 0;
    bool allzero = true;
    for (int i = 0; i < d; ++i) {
        size[i] = hi[i] - lo[i];
        biggest = std::max(biggest, size[i]);
        if (size[i] != 0) allzero = false;
    }
    for (int i = 0; i < d; ++i) size[i] = allzero ? 1.0 : (size[i] == 0 ? biggest : size[i]);
    code.assign((size_t)nelem * d, 0);
    for (int64_t e = 0; e < nelem; ++e) {
        uint64_t X[3];
        for (int i = 0; i < d; ++i) X[i] = scale_unit((centroids[e * d + i] - lo[i]) / size[i]);
        hilbert_code(X, d, 64, &code[(size_t)e * d]);
    }
}

static int bit_length(unsigned __int128 v) {
    int b = 0;
    while (v) {
        ++b;
        v >>= 1;
    }
    return b;
}

// The k-th of the n + 1 points of range(lo, stop = hi, length = n + 1):
// (lo (n - k) + hi k) / n rounded once to the nearest double (ties to even),
// computed exactly in 128-bit integers.  The centroid codes sit on dyadic
// boundaries for many bricks (a centroid at a quarter of the box), where
// one unit in the last place of a corner coordinate moves an element to
// another branch of the curve, so the corners must be the reference's
// range points to the last bit.
static double range_point(double lo, double hi, int n, int k) {
    if (k == 0) return lo;
    if (k == n) return hi;
    int el = 0, eh = 0;
    const double fl = std::frexp(lo, &el), fh = std::frexp(hi, &eh);
    const int64_t ml = (int64_t)std::ldexp(fl, 53), mh = (int64_t)std::ldexp(fh, 53);
    if (ml == 0) el = eh;
    if (mh == 0) eh = el;
    const int E = std::min(el, eh) - 53;  // lo = ml 2^(el - 53), hi = mh 2^(eh - 53)
    const int sl = el - 53 - E, sh = eh - 53 - E;
    if (sl > 40 || sh > 40)  // ends of very different magnitudes: extended precision
        return (double)(((long double)lo * (n - k) + (long double)hi * k) / n);
    const __int128 A = ((__int128)ml * (n - k)) * ((__int128)1 << sl) + ((__int128)mh * k) * ((__int128)1 << sh);
    if (A == 0) return 0.0;
    const bool neg = A < 0;
    const unsigned __int128 a = (unsigned __int128)(neg ? -A : A);
    const int nb = bit_length((unsigned __int128)n);
    const int shift = std::max(0, 56 + nb - bit_length(a));
    const unsigned __int128 num = a << shift;
    const unsigned __int128 Q = num / (unsigned)n, R = num % (unsigned)n;
    const int drop = bit_length(Q) - 53;  // >= 2: Q has at least 55 bits
    uint64_t mant = (uint64_t)(Q >> drop);
    const unsigned __int128 rest = Q & (((unsigned __int128)1 << drop) - 1), half = (unsigned __int128)1 << (drop - 1);
    if (rest > half || (rest == half && (R != 0 || (mant & 1u)))) ++mant;
    const double v = std::ldexp((double)mant, E - shift + drop);
    return neg ? -v : v;
}

// Hilbert order of the elements of a d-dimensional brick with ne[0..d-1]
// elements between lo and hi, created in Cartesian order (x fastest):
// order[p] = Cartesian index of the p-th element along the curve (ties, which
// only equal centroids can make, by Cartesian index).
static void brick_hilbert_order(const cmdg_brick_desc& b, int d, std::vector<int64_t>& order) {
    int64_t nelem = 1;
    for (int i = 0; i < d; ++i) nelem *= b.ne[i];
    std::vector<double> cent((size_t)nelem * d);
    for (int64_t e = 0; e < nelem; ++e) {
        int64_t r = e;
        for (int i = 0; i < d; ++i) {
            const int idx = (int)(r % b.ne[i]);
            r /= b.ne[i];
            // the corners' coordinates are the range's points; the centroid is
            // their sum (in corner order, 2^d terms) over 2^d
            const double a = range_point(b.lo[i], b.hi[i], b.ne[i], idx);
            const double c = range_point(b.lo[i], b.hi[i], b.ne[i], idx + 1);
            double s = 0;
            const int nvert = 1 << d;
            for (int v = 0; v < nvert; ++v) s += ((v >> i) & 1) ? c : a;
            cent[(size_t)e * d + i] = s / nvert;
        }
    }
    std::vector<uint64_t> code;
    centroid_codes(cent.data(), d, nelem, code);
    order.resize(nelem);
    std::iota(order.begin(), order.end(), 0);
    std::stable_sort(order.begin(), order.end(), [&](int64_t x, int64_t y) {
        for (int i = 0; i < d; ++i) {
            const uint64_t cx = code[(size_t)x * d + i], cy = code[(size_t)y * d + i];
            if (cx != cy) return cx < cy;
        }
        return false;
    });
}

// Column order of a brick mesh: for the StackedBrickTopology order the
// horizontal base elements along the 2D Hilbert curve, else x then y.
// col_at[h] = ix + nx iy of the h-th column.
int brick_column_order(const cmdg_brick_desc& b, int topology, std::vector<int>& col_at) {
    const int64_t ncol = (int64_t)b.ne[0] * b.ne[1];
    col_at.resize(ncol);
    if (topology == CMDG_TOPOLOGY_STACKED_BRICK) {
        std::vector<int64_t> order;
        brick_hilbert_order(b, 2, order);
        for (int64_t h = 0; h < ncol; ++h) col_at[h] = (int)order[h];
    } else {
        std::iota(col_at.begin(), col_at.end(), 0);
    }
    return CMDG_OK;
}

}  // namespace cmdg

using namespace cmdg;

extern "C" int cmdg_brick_element_order(const cmdg_brick_desc* desc, int topology, int64_t* h_perm) {
    CMDG_ARG_CHECK(desc != nullptr && h_perm != nullptr, "NULL argument");
    CMDG_ARG_CHECK(topology == CMDG_TOPOLOGY_LIBRARY || topology == CMDG_TOPOLOGY_BRICK ||
                       topology == CMDG_TOPOLOGY_STACKED_BRICK,
                   "unknown topology order %d", topology);
    for (int k = 0; k < 3; ++k) {
        CMDG_ARG_CHECK(desc->ne[k] >= 1, "ne[%d]=%d must be >= 1", k, desc->ne[k]);
        CMDG_ARG_CHECK(desc->hi[k] > desc->lo[k], "hi[%d] must exceed lo[%d]", k, k);
    }
    const int64_t nx = desc->ne[0], ny = desc->ne[1], nz = desc->ne[2];
    const int64_t nelem = nx * ny * nz;
    CMDG_ARG_CHECK(nelem < (int64_t)1 << 31, "too many elements (%lld)", (long long)nelem);
    auto lib = [&](int64_t ix, int64_t iy, int64_t iz) { return iz + nz * (ix + nx * iy); };
    if (topology == CMDG_TOPOLOGY_BRICK) {
        std::vector<int64_t> order;
        brick_hilbert_order(*desc, 3, order);
        for (int64_t p = 0; p < nelem; ++p) {
            const int64_t c = order[p];
            h_perm[p] = lib(c % nx, (c / nx) % ny, c / (nx * ny));
        }
        return CMDG_OK;
    }
    std::vector<int> col_at;
    brick_column_order(*desc, topology, col_at);
    for (int64_t h = 0; h < nx * ny; ++h)
        for (int64_t iz = 0; iz < nz; ++iz) h_perm[iz + nz * h] = lib(col_at[h] % nx, col_at[h] / nx, iz);
    return CMDG_OK;
}
