// harness.cpp — runs the reference project's own kernel sources
// (src/threshold.cpp, src/segmentation.cpp, src/find_boundaries.cpp,
// src/fit_quad.cpp, compiled from the reference tree against the host SYCL
// shim in include/sycl/sycl.hpp) and its record helpers (include/*.h) on one
// greyscale image, and writes every stage's output as raw little-endian
// arrays.  TEST INFRASTRUCTURE ONLY: golden-vector generation.
//
// Only the oneDPL glue of src/main.cpp (which needs oneDPL and cannot be
// compiled here) is restated, with the same tie orders as the oracle:
//   sort_by_key (main.cpp:515)          -> (key, packed point)
//   sort (cluster, slope) (:737)        -> (cluster, slope, packed point)
//   sort (cluster, error desc) (:857)   -> (cluster asc, error desc, index asc)
// The segmented scan of line-fit moments adds the int64 bit patterns as
// doubles, exactly as main.cpp:793-801 does.
//
// usage: harness <image.raw> <width> <height> <out_dir>
#include <sycl/sycl.hpp>

#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <string>
#include <vector>

#include "boundary_point.h"
#include "cluster_bounds.h"
#include "find_boundaries.h"
#include "fit_quad.h"
#include "line_fit_point.h"
#include "segmentation.h"
#include "threshold.h"

template <class T>
static void dump(const std::string& dir, const char* name, const T* data, size_t n) {
    std::string p = dir + "/" + name + ".bin";
    FILE* f = fopen(p.c_str(), "wb");
    if (!f) {
        perror(p.c_str());
        exit(1);
    }
    if (n) fwrite(data, sizeof(T), n, f);
    fclose(f);
}

static uint32_t as_u32(BoundaryPoint p) {
    uint32_t v;
    std::memcpy(&v, &p, 4);
    return v;
}

#include "combinadics.h"

// Deterministic generator for the record-helper vectors.
struct Lcg {
    uint64_t s;
    uint64_t next() {
        s = s * 6364136223846793005ull + 1442695040888963407ull;
        return s >> 17;
    }
    uint32_t below(uint32_t n) { return (uint32_t)(next() % n); }
};

// Evaluates the reference's record helpers (include/*.h, get_moment and
// fit_line of src/fit_quad.cpp) on seeded inputs and writes inputs and
// outputs side by side.
static int records(const std::string& out) {
    Lcg g{12345};
    // combinadics decode of every combination number do_indexing uses
    using C = Combinadics<uint8_t, 15, 4, 16>;
    std::vector<uint32_t> dec;
    for (uint32_t n = 0; n < 210; n++) {
        auto d = C::decode((uint8_t)n);
        for (int i = 0; i < 4; i++) dec.push_back((uint32_t)d[i]);
    }
    dump(out, "rec_combinadics", dec.data(), dec.size());
    // calc_theta against ClusterBounds::cx/cy; ValidBlobFilter and dot
    const int NB = 3000;
    std::vector<ClusterBounds> bs(NB);
    std::vector<BoundaryPoint> ps(NB);
    std::vector<float> theta(NB), cx(NB), cy(NB), dot(NB);
    std::vector<uint8_t> valid(NB);
    ValidBlobFilter filt(1920, 1080);
    for (int i = 0; i < NB; i++) {
        ClusterBounds b{};
        b.x_min = (uint16_t)g.below(8000);
        b.x_max = (uint16_t)(b.x_min + g.below(600));
        b.y_min = (uint16_t)g.below(4000);
        b.y_max = (uint16_t)(b.y_min + g.below(600));
        b.count = g.below(3) == 0 ? g.below(30) : g.below(20000);
        b.gx_sum = (int32_t)g.below(2 * b.count + 1) - (int32_t)b.count;
        b.gy_sum = 0;
        b.pxgx_pygy_sum = (int64_t)g.below(2000000000) - 1000000000;
        b.start = g.below(1 << 20);
        bs[i] = b;
        BoundaryPoint p{(uint16_t)(g.below(4096) | (g.below(4) << 14)), (uint16_t)(g.below(4096) | (g.below(2) << 15))};
        ps[i] = p;
        cx[i] = b.cx();
        cy[i] = b.cy();
        theta[i] = p.calc_theta(cx[i], cy[i]);
        dot[i] = b.dot();
        valid[i] = filt(b);
    }
    dump(out, "rec_bounds", bs.data(), NB);
    dump(out, "rec_points", ps.data(), NB);
    dump(out, "rec_cx", cx.data(), NB);
    dump(out, "rec_cy", cy.data(), NB);
    dump(out, "rec_theta", theta.data(), NB);
    dump(out, "rec_dot", dot.data(), NB);
    dump(out, "rec_valid", valid.data(), NB);
    // compute_initial_linefit on a random image
    const uint32_t W = 256, H = 192;
    std::vector<uint8_t> img(W * H);
    for (auto& v : img) v = (uint8_t)g.below(256);
    std::vector<ClusterPoint> cps(NB);
    std::vector<LineFitPoint> lfs(NB);
    for (int i = 0; i < NB; i++) {
        cps[i] = ClusterPoint{(uint16_t)(g.below(W + 4) | (g.below(4) << 14)), (uint16_t)(g.below(H + 4) | (g.below(2) << 15)), 0.0f};
        lfs[i] = compute_initial_linefit(cps[i], W, H, img.data());
        lfs[i].a = lfs[i].b = 0;
    }
    dump(out, "rec_image", img.data(), img.size());
    dump(out, "rec_cluster_points", cps.data(), NB);
    dump(out, "rec_linefit", lfs.data(), NB);
    // fit_line on moments of random point sets, plus wrapped extremes
    std::vector<LineFitPoint> ms(NB);
    std::vector<uint64_t> nim(NB);
    std::vector<float> lp(4 * NB), err(NB), mse(NB);
    for (int i = 0; i < NB; i++) {
        LineFitPoint m{};
        int n = 1 + (int)g.below(200);
        int64_t x0 = g.below(8000), y0 = g.below(8000);
        int64_t dx = (int64_t)g.below(9) - 4, dy = (int64_t)g.below(9) - 4;
        for (int k = 0; k < n; k++) {
            int64_t W8 = 1 + g.below(300);
            int64_t rx = x0 + dx * k + g.below(3), ry = y0 + dy * k + g.below(3);
            m.Mx += W8 * rx; m.My += W8 * ry; m.Mxx += W8 * rx * rx; m.Myy += W8 * ry * ry; m.Mxy += W8 * rx * ry;
            m.W += W8;
        }
        if (i % 97 == 0) {  // products that overflow int64 on purpose
            m.Mxx = (int64_t)(g.next() << 20); m.Mxy = (int64_t)(g.next() << 21); m.W = (int64_t)(1 + g.below(1 << 30));
        }
        ms[i] = m;
        nim[i] = (uint64_t)n + (i % 113 == 0 ? (uint64_t)-5 : 0);
        fit_line(m, nim[i], &lp[4 * i], &err[i], &mse[i]);
    }
    dump(out, "rec_moments", ms.data(), NB);
    dump(out, "rec_num_in_moment", nim.data(), NB);
    dump(out, "rec_line_params", lp.data(), 4 * NB);
    dump(out, "rec_err", err.data(), NB);
    dump(out, "rec_mse", mse.data(), NB);
    // get_moment over a prefix array, including the wrapping (i1 < i0) case
    const int NP = 500;
    std::vector<LineFitPoint> pre(NP);
    LineFitPoint acc{};
    for (int i = 0; i < NP; i++) {
        LineFitPoint one = compute_initial_linefit(cps[i], W, H, img.data());
        acc += one;
        acc.a = acc.b = 0;
        pre[i] = acc;
    }
    std::vector<uint64_t> gi(2 * NB), gn(NB);
    std::vector<LineFitPoint> gm(NB);
    for (int i = 0; i < NB; i++) {
        size_t i0 = g.below(NP), i1 = g.below(NP);
        if (i0 == 0 && i1 < i0) i0 = 1;
        auto [m, n] = get_moment(pre.data(), NP, i0, i1);
        m.a = m.b = 0;
        gi[2 * i] = i0; gi[2 * i + 1] = i1; gm[i] = m; gn[i] = n;
    }
    dump(out, "rec_prefix", pre.data(), NP);
    dump(out, "rec_moment_range", gi.data(), 2 * NB);
    dump(out, "rec_moment", gm.data(), NB);
    dump(out, "rec_moment_n", gn.data(), NB);
    printf("records ok\n");
    return 0;
}

int main(int argc, char** argv) {
    if (argc == 3 && std::string(argv[1]) == "--records") return records(argv[2]);
    if (argc != 5) {
        fprintf(stderr, "usage: %s image.raw width height out_dir\n", argv[0]);
        return 2;
    }
    const size_t w = std::stoul(argv[2]), h = std::stoul(argv[3]), N = w * h;
    const std::string out = argv[4];
    std::vector<uint8_t> grey(N);
    FILE* f = fopen(argv[1], "rb");
    if (!f || fread(grey.data(), 1, N, f) != N) {
        fprintf(stderr, "cannot read %s\n", argv[1]);
        return 1;
    }
    fclose(f);
    sycl::queue q;

    // stage 1: threshold_image
    std::vector<sycl::vec<uint8_t, 2>> extrema(N / 16), filtered(N / 16);
    std::vector<uint8_t> thr(N);
    threshold_image(q, grey.data(), extrema.data(), filtered.data(), thr.data(), w, h).wait();
    dump(out, "thresholded", thr.data(), N);
    dump(out, "extrema", extrema.data(), N / 16);
    dump(out, "filtered_extrema", filtered.data(), N / 16);

    // stage 2: image_segmentation (all N sizes zeroed, see main.cpp:311)
    std::vector<uint32_t> scratch(N), labels(N), sizes(N, 0);
    image_segmentation(q, thr.data(), scratch.data(), labels.data(), sizes.data(), 1 << 16, w, h).wait();
    dump(out, "labels", labels.data(), N);
    dump(out, "sizes", sizes.data(), N);

    // stage 3: find_boundaries into pre-filled dense planes (main.cpp:312-315)
    std::vector<BoundaryPoint> dpts(4 * N);
    std::vector<uint64_t> dkeys(4 * N, ~0ull);
    std::memset(dpts.data(), 0, dpts.size() * sizeof(BoundaryPoint));
    find_boundaries(q, labels.data(), sizes.data(), dpts.data(), dkeys.data(), w, h).wait();
    dump(out, "dense_points", dpts.data(), 4 * N);
    dump(out, "dense_keys", dkeys.data(), 4 * N);

    // stage 4-5: copy_if + sort_by_key
    struct KP {
        uint64_t key;
        BoundaryPoint p;
    };
    std::vector<KP> kp;
    for (size_t i = 0; i < 4 * N; i++)
        if (as_u32(dpts[i]) != 0) kp.push_back({dkeys[i], dpts[i]});
    std::sort(kp.begin(), kp.end(), [](const KP& a, const KP& b) {
        if (a.key != b.key) return a.key < b.key;
        return as_u32(a.p) < as_u32(b.p);
    });
    const size_t P = kp.size();
    std::vector<BoundaryPoint> pts(P);
    std::vector<uint64_t> keys(P);
    for (size_t i = 0; i < P; i++) {
        pts[i] = kp[i].p;
        keys[i] = kp[i].key;
    }
    dump(out, "points", pts.data(), P);
    dump(out, "keys", keys.data(), P);

    // stage 6: reduce_by_segment -> ClusterBounds
    std::vector<ClusterBounds> bounds;
    std::vector<uint64_t> bound_keys;
    for (size_t i = 0; i < P; i++) {
        ClusterBounds b = ClusterBounds::inital_from_point(pts[i], (uint32_t)i);
        if (i == 0 || keys[i] != keys[i - 1]) {
            bounds.push_back(b);
            bound_keys.push_back(keys[i]);
        } else {
            bounds.back() = reduce_bounds(bounds.back(), b);
        }
    }
    dump(out, "bounds", bounds.data(), bounds.size());
    dump(out, "bound_keys", bound_keys.data(), bound_keys.size());

    // stage 6b: ValidBlobFilter
    ValidBlobFilter filter(w, h);
    std::vector<ClusterBounds> fb;
    std::vector<uint64_t> fkeys;
    for (size_t c = 0; c < bounds.size(); c++)
        if (filter(bounds[c])) {
            fb.push_back(bounds[c]);
            fkeys.push_back(bound_keys[c]);
        }
    dump(out, "filtered_bounds", fb.data(), fb.size());
    dump(out, "filtered_keys", fkeys.data(), fkeys.size());

    // stage 7: points -> clusters + theta (main.cpp:621-675)
    struct CP {
        ClusterPoint p;
        uint16_t c;
    };
    std::vector<CP> cps;
    for (uint32_t i = 0; i < P; i++) {
        auto it = std::lower_bound(fb.begin(), fb.end(), i,
                                   [](const ClusterBounds& a, uint32_t b) { return (a.start + a.count) <= b; });
        if (it == fb.end()) continue;
        if (i < it->start || i >= it->start + it->count) continue;
        BoundaryPoint bp = pts[i];
        cps.push_back({ClusterPoint{bp.packed_x, bp.packed_y, bp.calc_theta(it->cx(), it->cy())},
                       (uint16_t)std::distance(fb.begin(), it)});
    }
    // stage 8: extents
    std::vector<ClusterExtents> extents(fb.size());
    {
        uint32_t s = 0;
        for (size_t c = 0; c < fb.size(); c++) {
            extents[c] = ClusterExtents{s, fb[c].count};
            s += fb[c].count;
        }
    }
    dump(out, "extents", extents.data(), extents.size());
    // stage 9: sort by (cluster, slope)
    auto cpu = [](const ClusterPoint& p) {
        uint32_t v = (uint32_t)p.packed_x | ((uint32_t)p.packed_y << 16);
        return v;
    };
    std::sort(cps.begin(), cps.end(), [&](const CP& a, const CP& b) {
        if (a.c != b.c) return a.c < b.c;
        if (a.p.slope < b.p.slope) return true;
        if (b.p.slope < a.p.slope) return false;
        return cpu(a.p) < cpu(b.p);
    });
    const size_t Pf = cps.size();
    std::vector<ClusterPoint> cpts(Pf);
    std::vector<uint16_t> cidx(Pf);
    for (size_t i = 0; i < Pf; i++) {
        cpts[i] = cps[i].p;
        cidx[i] = cps[i].c;
    }
    dump(out, "cluster_points", cpts.data(), Pf);
    dump(out, "cluster_indices", cidx.data(), Pf);

    // stage 10: compute_initial_linefit; stage 11: segmented scan as doubles
    std::vector<LineFitPoint> lf(Pf);
    for (size_t i = 0; i < Pf; i++) {
        lf[i] = compute_initial_linefit(cpts[i], (uint32_t)w, (uint32_t)h, grey.data());
        lf[i].a = 0;
        lf[i].b = 0;
    }
    for (size_t i = 1; i < Pf; i++) {
        if (cidx[i] != cidx[i - 1]) continue;
        double a[8], b[8];
        std::memcpy(a, &lf[i - 1], 64);
        std::memcpy(b, &lf[i], 64);
        for (int k = 0; k < 8; k++) b[k] = a[k] + b[k];
        std::memcpy(&lf[i], b, 64);
    }
    dump(out, "line_fit", lf.data(), Pf);

    // stage 12: fit_lines (reference kernel), pre-zeroed output
    std::vector<Corner> found(Pf);
    std::memset(found.data(), 0, found.size() * sizeof(Corner));
    if (Pf) fit_lines(q, lf.data(), cidx.data(), extents.data(), Pf, found.data());
    dump(out, "found_corners", found.data(), Pf);

    // stages 13-15: copy_if (error != 0), sort, reduce_by_segment
    std::vector<Corner> corners;
    for (const Corner& c : found)
        if (c.error != 0) corners.push_back(c);
    std::sort(corners.begin(), corners.end(), [](const Corner& a, const Corner& b) {
        if (a.cluster_index != b.cluster_index) return a.cluster_index < b.cluster_index;
        if (a.error > b.error) return true;
        if (b.error > a.error) return false;
        return a.line_fit_point_index < b.line_fit_point_index;
    });
    dump(out, "corners", corners.data(), corners.size());
    std::vector<PeakExtents> pe;
    for (size_t i = 0; i < corners.size(); i++) {
        PeakExtents e{(uint32_t)i, 1};
        if (i == 0 || corners[i].cluster_index != corners[i - 1].cluster_index)
            pe.push_back(e);
        else
            pe.back() = reduce_extents(pe.back(), e);
    }
    dump(out, "peak_extents", pe.data(), pe.size());

    // stage 16: do_indexing (reference kernel), pre-zeroed output
    std::vector<FittedQuad> fitted(pe.size());
    std::memset(fitted.data(), 0, fitted.size() * sizeof(FittedQuad));
    if (!pe.empty()) do_indexing(q, pe.data(), pe.size(), corners.data(), lf.data(), extents.data(), fitted.data());
    dump(out, "fitted", fitted.data(), fitted.size());

    // process_fitted_quads (main.cpp:1035-1162) up to decoding, restated
    // around the reference's fit_line; QuadCorners.blob_index is set to the
    // FittedQuad's position (the reference leaves it unset).
    std::vector<QuadCorners> quads;
    const int min_tag_width_ = 8;
    const double cos_critical_rad = std::cos(10 * M_PI / 180);
    for (size_t qi = 0; qi < fitted.size(); qi++) {
        const FittedQuad& quad = fitted[qi];
        if (!(quad.indices[0] != 0 || quad.indices[1] != 0 || quad.indices[2] != 0 || quad.indices[3] != 0)) continue;
        QuadCorners corners_out;
        std::memset(&corners_out, 0, sizeof corners_out);
        corners_out.reversed_border = false;
        corners_out.blob_index = (uint32_t)qi;
        float lines[4][4];
        for (int i = 0; i < 4; i++) {
            float err, mse;
            fit_line(quad.moments[i], quad.num_in_moments[i], lines[i], &err, &mse);
        }
        bool bad = false;
        for (int i = 0; i < 4; i++) {
            double A00 = lines[i][3], A01 = -lines[(i + 1) & 3][3];
            double A10 = -lines[i][2], A11 = lines[(i + 1) & 3][2];
            double B0 = -lines[i][0] + lines[(i + 1) & 3][0];
            double B1 = -lines[i][1] + lines[(i + 1) & 3][1];
            double det = A00 * A11 - A10 * A01;
            double W00 = A11 / det, W01 = -A01 / det;
            if (fabs(det) < 0.001) {
                bad = true;
                break;
            }
            double L0 = W00 * B0 + W01 * B1;
            corners_out.corners[i][0] = lines[i][0] + L0 * A00;
            corners_out.corners[i][1] = lines[i][1] + L0 * A10;
        }
        if (bad) continue;
        {
            float area = 0, length[3], p;
            for (int i = 0; i < 3; i++) {
                int a = i, b = (i + 1) % 3;
                length[i] = hypotf(corners_out.corners[b][0] - corners_out.corners[a][0],
                                   corners_out.corners[b][1] - corners_out.corners[a][1]);
            }
            p = (length[0] + length[1] + length[2]) / 2;
            area += sqrtf(p * (p - length[0]) * (p - length[1]) * (p - length[2]));
            for (int i = 0; i < 3; i++) {
                int idxs[] = {2, 3, 0, 2};
                int a = idxs[i], b = idxs[i + 1];
                length[i] = hypotf(corners_out.corners[b][0] - corners_out.corners[a][0],
                                   corners_out.corners[b][1] - corners_out.corners[a][1]);
            }
            p = (length[0] + length[1] + length[2]) / 2;
            area += sqrtf(p * (p - length[0]) * (p - length[1]) * (p - length[2]));
            if (area < 0.95 * min_tag_width_ * min_tag_width_) continue;
        }
        bool reject = false;
        for (int i = 0; i < 4; i++) {
            int i0 = i, i1 = (i + 1) & 3, i2 = (i + 2) & 3;
            float dx1 = corners_out.corners[i1][0] - corners_out.corners[i0][0];
            float dy1 = corners_out.corners[i1][1] - corners_out.corners[i0][1];
            float dx2 = corners_out.corners[i2][0] - corners_out.corners[i1][0];
            float dy2 = corners_out.corners[i2][1] - corners_out.corners[i1][1];
            float cos_dtheta = (dx1 * dx2 + dy1 * dy2) / sqrtf((dx1 * dx1 + dy1 * dy1) * (dx2 * dx2 + dy2 * dy2));
            if (std::abs(cos_dtheta) > cos_critical_rad || dx1 * dy2 < dy1 * dx2) {
                reject = true;
                break;
            }
        }
        if (reject) continue;
        quads.push_back(corners_out);
    }
    dump(out, "quads", quads.data(), quads.size());
    printf("P=%zu C=%zu Cf=%zu Pf=%zu K=%zu Cp=%zu Q=%zu\n", P, bounds.size(), fb.size(), Pf, corners.size(),
           pe.size(), quads.size());
    return 0;
}
