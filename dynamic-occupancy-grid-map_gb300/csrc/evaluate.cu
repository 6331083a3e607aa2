// Accuracy evaluation of the dynamic cells against ground-truth objects (host code).
//
// Restates the demo's evaluator (dogm/demo/utils/precision_evaluator.cpp:16-139, dbscan.cpp,
// metrics.cpp): the dynamic cells of a frame are clustered by DBSCAN (neighbour distance 3 cells,
// at least 5 neighbours counting the cell itself, precision_evaluator.cpp:16-18); each cluster's
// mean position and velocity, in metres with y pointing up (precision_evaluator.cpp:98-121), is
// assigned to the nearest ground-truth object closer than 5 m (precision_evaluator.cpp:49-77),
// and the position and velocity errors accumulate into a mean absolute error and a
// root-mean-square error (metrics.cpp:8-56).  Clusters matched by no object count as
// unassigned detections.
//
// Two clustering modes.  DOGM_DBSCAN_REFERENCE reproduces dbscan.cpp:55-98 exactly, including
// its labelling slip: when a core point starts a cluster, expandCluster labels the first |seeds|
// points of the input (dbscan.cpp:64-67) rather than the seeds, so early points can move between
// clusters, a cluster can end up empty (its mean is NaN, and it counts as unassigned, as in the
// reference), and the starting point stays unlabelled unless a core neighbour reaches it.
// DOGM_DBSCAN_STANDARD is the published algorithm (Ester et al., KDD 1996) with the same visiting
// order.  Both grow a cluster from a queue of seeds; which points end up labelled does not depend
// on the queue order, so region queries can come from a hash of eps-sized buckets instead of a
// scan of every point.  Coordinates are assumed distinct (one entry per grid cell).
//
// Floating point follows the reference: distances are sqrtf(dx*dx + dy*dy) compared with <= eps
// and < 5 m, cluster sums are float sums in input order, error sums are float sums in cluster
// order, and the host compiler contracts no multiply-add.
#include <algorithm>
#include <cmath>
#include <cstdint>
#include <deque>
#include <unordered_map>
#include <vector>

#include "dogm_internal.h"

using namespace dogm_gb300;

namespace {

constexpr int kUnclassified = -2, kNoise = -1;

struct Points {
    std::vector<float> x, y;
    std::unordered_map<long long, std::vector<int>> bucket;
    float size = 1.f, eps = 1.f;

    static long long key(long long bx, long long by) { return (bx << 32) ^ (by & 0xffffffffll); }

    Points(const dogm_dynamic_cell* c, int n, float e) : x(n), y(n), size(e), eps(e) {
        for (int i = 0; i < n; ++i) {
            x[i] = c[i].x;
            y[i] = c[i].y;
            bucket[key((long long)std::floor(x[i] / size), (long long)std::floor(y[i] / size))].push_back(i);
        }
    }

    // Indices within eps of point q (q included), ascending.
    void region(int q, std::vector<int>& out) const {
        out.clear();
        const long long bx = (long long)std::floor(x[q] / size), by = (long long)std::floor(y[q] / size);
        for (long long dx = -1; dx <= 1; ++dx)
            for (long long dy = -1; dy <= 1; ++dy) {
                auto it = bucket.find(key(bx + dx, by + dy));
                if (it == bucket.end()) continue;
                for (int p : it->second) {
                    const float ddx = x[q] - x[p], ddy = y[q] - y[p];
                    const float sq = ddx * ddx + ddy * ddy;
                    if (std::sqrt(sq) <= eps) out.push_back(p);
                }
            }
        std::sort(out.begin(), out.end());
    }
};

// Returns the number of clusters; label[i] = cluster, or -1 for noise / no cluster.
int dbscan(const Points& pts, int min_cells, int mode, std::vector<int>& label) {
    const int n = (int)pts.x.size();
    label.assign(n, kUnclassified);
    std::vector<int> seen(n, -1);  // cluster in which a point was last taken from the queue
    std::vector<int> nb, nb2;
    std::deque<int> seeds;
    int cluster = 0;
    for (int i = 0; i < n; ++i) {
        if (label[i] != kUnclassified) continue;
        pts.region(i, nb);
        if ((int)nb.size() < min_cells) {
            label[i] = kNoise;
            continue;
        }
        seeds.clear();
        if (mode == DOGM_DBSCAN_REFERENCE) {
            for (int k = 0; k < (int)nb.size(); ++k) label[k] = cluster;  // dbscan.cpp:64-67
            for (int p : nb)
                if (p != i) seeds.push_back(p);
        } else {
            label[i] = cluster;
            for (int p : nb)
                if (p != i && (label[p] == kUnclassified || label[p] == kNoise)) {
                    if (label[p] == kUnclassified) seeds.push_back(p);
                    label[p] = cluster;
                }
        }
        while (!seeds.empty()) {
            const int c = seeds.front();
            seeds.pop_front();
            if (seen[c] == cluster) continue;  // a second visit changes no label
            seen[c] = cluster;
            pts.region(c, nb2);
            if ((int)nb2.size() < min_cells) continue;
            for (int p : nb2)
                if (label[p] == kUnclassified || label[p] == kNoise) {
                    if (label[p] == kUnclassified) seeds.push_back(p);
                    label[p] = cluster;
                }
        }
        ++cluster;
    }
    for (int& l : label)
        if (l < 0) l = -1;
    return cluster;
}

}  // namespace

struct dogm_evaluator {
    float resolution, grid_length, max_assign, eps;
    int min_cells, mode;
    float abs_err[4] = {0, 0, 0, 0}, sq_err[4] = {0, 0, 0, 0};
    int detections = 0, unassigned = 0;
};

extern "C" {

dogm_status dogm_cluster_cells(const dogm_dynamic_cell* cells, int n, float eps, int min_cells, int mode,
                               int* label, int* n_clusters) {
    if (n < 0 || (n > 0 && (!cells || !label)) || !n_clusters || !(eps > 0.f) || min_cells < 1 ||
        (mode != DOGM_DBSCAN_REFERENCE && mode != DOGM_DBSCAN_STANDARD)) {
        set_last_error("dogm_cluster_cells: bad argument");
        return DOGM_ERR_INVALID_ARGUMENT;
    }
    Points pts(cells, n, eps);
    std::vector<int> lab;
    *n_clusters = dbscan(pts, min_cells, mode, lab);
    std::copy(lab.begin(), lab.end(), label);
    return DOGM_OK;
}

dogm_status dogm_evaluator_create(float resolution, float grid_length, int dbscan_mode, dogm_evaluator** out) {
    if (!out || !(resolution > 0.f) || !(grid_length > 0.f) ||
        (dbscan_mode != DOGM_DBSCAN_REFERENCE && dbscan_mode != DOGM_DBSCAN_STANDARD)) {
        set_last_error("dogm_evaluator_create: bad argument");
        return DOGM_ERR_INVALID_ARGUMENT;
    }
    dogm_evaluator* e = new dogm_evaluator();
    e->resolution = resolution;
    e->grid_length = grid_length;
    e->max_assign = 5.0f;  // kMaximumAssignmentDistance
    e->eps = 3.0f;         // kMaximumDbscanNeighborDistance
    e->min_cells = 5;      // kMinimumNumberOfNeighbors
    e->mode = dbscan_mode;
    *out = e;
    return DOGM_OK;
}

dogm_status dogm_evaluator_destroy(dogm_evaluator* e) {
    delete e;
    return DOGM_OK;
}

dogm_status dogm_evaluator_add_step(dogm_evaluator* e, const dogm_dynamic_cell* cells, int n,
                                    const dogm_object_truth* truth, int n_truth, dogm_cluster* clusters,
                                    int max_clusters, int* n_clusters) {
    if (!e || n < 0 || n_truth < 0 || (n > 0 && !cells) || (n_truth > 0 && !truth) || !n_clusters ||
        (max_clusters > 0 && !clusters)) {
        set_last_error("dogm_evaluator_add_step: bad argument");
        return DOGM_ERR_INVALID_ARGUMENT;
    }
    *n_clusters = 0;
    if (n == 0 || n_truth == 0) return DOGM_OK;  // precision_evaluator.cpp:42
    Points pts(cells, n, e->eps);
    std::vector<int> label;
    const int nc = dbscan(pts, e->min_cells, e->mode, label);
    std::vector<float> sx(nc, 0.f), sy(nc, 0.f), svx(nc, 0.f), svy(nc, 0.f);
    std::vector<int> cnt(nc, 0);
    for (int i = 0; i < n; ++i) {
        const int c = label[i];
        if (c < 0) continue;
        sx[c] += cells[i].x;
        sy[c] += cells[i].y;
        svx[c] += cells[i].cell.mean_x_vel;
        svy[c] += cells[i].cell.mean_y_vel;
        cnt[c] += 1;
    }
    for (int c = 0; c < nc; ++c) {
        const float k = (float)cnt[c];  // 0 for a cluster emptied by the reference's slip: NaN mean
        dogm_cluster d{};
        d.x = (sx[c] / k) * e->resolution;
        d.y = e->grid_length - (sy[c] / k) * e->resolution;  // rows run down, y runs up
        d.vx = (svx[c] / k) * e->resolution;
        d.vy = -((svy[c] / k) * e->resolution);
        d.cells = cnt[c];
        d.truth = -1;
        float best = 0.f;
        for (int t = 0; t < n_truth; ++t) {
            const float dx = d.x - truth[t].x, dy = d.y - truth[t].y;
            const float sq = dx * dx + dy * dy;
            const float dist = std::sqrt(sq);
            if (dist < e->max_assign && (d.truth < 0 || dist < best)) {
                d.truth = t;
                best = dist;
            }
        }
        if (d.truth < 0) {
            e->unassigned += 1;
        } else {
            const dogm_object_truth& v = truth[d.truth];
            d.err_x = d.x - v.x;
            d.err_y = d.y - v.y;
            d.err_vx = d.vx - v.vx;
            d.err_vy = d.vy - v.vy;
            const float errs[4] = {d.err_x, d.err_y, d.err_vx, d.err_vy};
            for (int j = 0; j < 4; ++j) {
                e->abs_err[j] += std::fabs(errs[j]);
                const float sq = errs[j] * errs[j];
                e->sq_err[j] += sq;
            }
            e->detections += 1;
        }
        if (c < max_clusters) clusters[c] = d;
    }
    *n_clusters = nc;
    return DOGM_OK;
}

dogm_status dogm_evaluator_summary(const dogm_evaluator* e, float* mae4, float* rmse4, int* detections,
                                   int* unassigned) {
    if (!e) {
        set_last_error("dogm_evaluator_summary: evaluator is NULL");
        return DOGM_ERR_INVALID_ARGUMENT;
    }
    // metrics.cpp:22-31 and 47-56: float sums over an int count (0/0 gives NaN, as there)
    for (int j = 0; j < 4; ++j) {
        if (mae4) mae4[j] = e->abs_err[j] / (float)e->detections;
        if (rmse4) rmse4[j] = std::sqrt(e->sq_err[j] / (float)e->detections);
    }
    if (detections) *detections = e->detections;
    if (unassigned) *unassigned = e->unassigned;
    return DOGM_OK;
}

}  // extern "C"
