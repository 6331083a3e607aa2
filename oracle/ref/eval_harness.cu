// Reference-evaluator harness (test infrastructure: the checker, not the product).
//
// Linked with the reference's own demo evaluator sources, compiled where they lie
// (dogm/demo/utils/dbscan.cpp, metrics.cpp, precision_evaluator.cpp; see oracle/ref/build_ref.py),
// it exposes two C entry points so the tests can feed the same cells and objects to the
// reference and to dogm_cluster_cells / dogm_evaluator_*:
//   ref_dbscan    DBSCAN<dogm::GridCell>::cluster over points (x, y); label[i] = the index of the
//                 cluster holding point i, -1 if none.
//   ref_evaluate  PrecisionEvaluator with an MAE and an RMSE metric over `steps` frames; writes
//                 both statistics and the unassigned-detection count printSummary reports.
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <iostream>
#include <memory>
#include <sstream>
#include <string>
#include <vector>

#include "dbscan.h"
#include "metrics.h"
#include "precision_evaluator.h"

namespace {

std::vector<Point<dogm::GridCell>> make_points(const float* x, const float* y, const float* vx, const float* vy,
                                               int n) {
    std::vector<Point<dogm::GridCell>> pts(n);
    for (int i = 0; i < n; ++i) {
        Point<dogm::GridCell> p{};
        p.x = x[i];
        p.y = y[i];
        p.data = dogm::GridCell{};
        if (vx) p.data.mean_x_vel = vx[i];
        if (vy) p.data.mean_y_vel = vy[i];
        p.cluster_id = UNCLASSIFIED;
        pts[i] = p;
    }
    return pts;
}

}  // namespace

extern "C" int ref_dbscan(const float* x, const float* y, int n, float eps, int min_cells, int* label) {
    const auto pts = make_points(x, y, nullptr, nullptr, n);
    const DBSCAN<dogm::GridCell> dbscan(eps, min_cells);
    const Clusters<dogm::GridCell> clusters = dbscan.cluster(pts);
    for (int i = 0; i < n; ++i) label[i] = -1;
    for (int c = 0; c < (int)clusters.size(); ++c)
        for (const auto& p : clusters[c])
            for (int i = 0; i < n; ++i)
                if (x[i] == p.x && y[i] == p.y) label[i] = c;
    return (int)clusters.size();
}

// cell_off / truth_off: steps + 1 offsets into the concatenated per-frame arrays.
extern "C" int ref_evaluate(int steps, const int* cell_off, const float* cx, const float* cy, const float* cvx,
                            const float* cvy, const int* truth_off, const float* tx, const float* ty,
                            const float* tvx, const float* tvy, float resolution, float grid_size, float* mae4,
                            float* rmse4, int* unassigned) {
    SimulationData sim(steps);
    for (int s = 0; s < steps; ++s)
        for (int t = truth_off[s]; t < truth_off[s + 1]; ++t)
            sim[s].vehicles.push_back(Vehicle(1.0f, glm::vec2(tx[t], ty[t]), glm::vec2(tvx[t], tvy[t])));
    PrecisionEvaluator evaluator(sim, resolution, grid_size);
    auto mae = std::make_unique<MAE>();
    auto rmse = std::make_unique<RMSE>();
    MAE* mae_p = mae.get();
    RMSE* rmse_p = rmse.get();
    evaluator.registerMetric("MAE", std::move(mae));
    evaluator.registerMetric("RMSE", std::move(rmse));
    for (int s = 0; s < steps; ++s) {
        const int a = cell_off[s], n = cell_off[s + 1] - a;
        evaluator.evaluateAndStoreStep(s, make_points(cx + a, cy + a, cvx + a, cvy + a, n));
    }
    const PointWithVelocity m = mae_p->computeErrorStatistic();
    const PointWithVelocity r = rmse_p->computeErrorStatistic();
    const float mv[4] = {m.x, m.y, m.v_x, m.v_y}, rv[4] = {r.x, r.y, r.v_x, r.v_y};
    std::memcpy(mae4, mv, sizeof(mv));
    std::memcpy(rmse4, rv, sizeof(rv));
    // the unassigned count is private to PrecisionEvaluator; printSummary reports it
    std::ostringstream text;
    std::streambuf* old = std::cout.rdbuf(text.rdbuf());
    evaluator.printSummary();
    std::cout.rdbuf(old);
    const std::string s = text.str();
    const std::string key = "Detections unassigned by evaluator: ";
    const size_t at = s.find(key);
    *unassigned = at == std::string::npos ? -1 : std::atoi(s.c_str() + at + key.size());
    return 0;
}
