// Host planner: reproduces the KernelMatrix block tree of HierarchicalMatrices.jl
// (src/KernelMatrix.jl:47-116 with indsplit, src/BarycentricMatrix.jl:299-307)
// and flattens it into the device tables of hm_types.h.
#pragma once
#include <stdint.h>
#include <vector>

#include "hm_types.h"

namespace hm {

enum PlanStatus {
    PLAN_OK = 0,
    PLAN_ERR_BOUNDS = 3,        // the reference would raise BoundsError in indsplit
    PLAN_ERR_DEGENERATE = 9,    // a partition the reference builds inconsistently
};

struct Node {
    int64_t lo, hi;     // [lo, hi) 0-based indices into the point list
    double a, b;        // box; children are [a, (a+b)/2] and [(a+b)/2, b]
    int level;
    int parent;
    int child[2];
    bool used;          // cluster of at least one barycentric block
    bool sub_used;      // some strict descendant is used
    int kind;           // 0 none, 1 internal basis node, 2 basis leaf
    int slot;           // coefficient slot, -1 if none
};

struct Tree {
    const double *x = nullptr;
    int64_t n = 0;
    std::vector<Node> nodes;
    void init(const double *pts, int64_t npts, double a, double b);
    // Computes the children of node id once (indsplit semantics).
    int split(int id);
    int64_t size(int id) const { return nodes[id].hi - nodes[id].lo; }
};

struct PlanStats {
    int64_t n_bary = 0, n_dense = 0, depth = 0;
    int64_t n_xslots = 0, n_yslots = 0;
    int64_t canonical_values = 0;   // cluster-deduplicated U, V + F + dense leaves
    int64_t reference_values = 0;   // per-block U, V, F + dense (the reference's layout)
    int64_t stored_values = 0;      // what this plan stores (nested bases)
    int64_t dense_values = 0;
    int64_t n_segments = 0;
    int64_t max_width = 0;
};

struct Plan {
    int r = 0;
    int64_t nx = 0, ny = 0;
    Tree X, Y;
    std::vector<std::pair<int, int>> bary;    // (x node, y node)
    std::vector<std::pair<int, int>> dense;   // (x node, y node)

    // flattened tables
    std::vector<hm_vpanel> vpanels;           // y-side explicit bases
    std::vector<hm_fill_vpanel> vpanel_fill;
    int64_t vstore_elems = 0;
    std::vector<hm_xfer> up;                  // y tree, deepest level first
    std::vector<int> up_level_ptr;            // ranges of `up` per level step
    std::vector<hm_m2l_row> m2l_rows;
    std::vector<hm_m2l_ent> m2l_ents;
    std::vector<hm_fill_f> f_fill;
    int64_t fstore_elems = 0;
    int fstride = 0;                          // elements between F blocks (r*r rounded to 4)
    // banded transfers (records ordered band by band, task by task, step by step)
    std::vector<hm_xfer> up_ents, down_ents;
    std::vector<hm_step> up_steps, down_steps;
    std::vector<hm_task> up_tasks, down_tasks;
    std::vector<int> up_band_ptr, down_band_ptr;   // task ranges per band, in launch order
    std::vector<hm_xfer> down;                // x tree, top level first
    std::vector<int> down_level_ptr;
    std::vector<hm_seg> segs;
    std::vector<hm_piece> pieces;
    std::vector<hm_fill_seg> seg_fill;
    int64_t pstore_elems = 0;
    int n_xslots = 0, n_yslots = 0;
    int max_width = 0;
    PlanStats stats;
};

// Builds the plan.  x, y must be non-increasing (validated by the caller);
// leaf = BLOCKSIZE, r = rank, seg_rows = maximum rows per row segment.
int build_plan(const double *x, int64_t nx, const double *y, int64_t ny, double a, double b,
               double c, double d, int r, int64_t leaf, int seg_rows, Plan &out);

constexpr int kBandLevels = 4;   // tree levels per transfer band

// A user-assembled HierarchicalMatrix flattened to leaf blocks (the block
// walk of src/HierarchicalMatrix.jl:24-52 gives each leaf its row and column
// offsets).  kind 0: dense A (rows x cols, column-major); kind 1: LowRankMatrix
// U diag(sigma) V^T (src/LowRankMatrix.jl:28-33; U rows x r, sigma r, V cols x r,
// contiguous); kind 2: U C V^T with an r x r core C (a BarycentricMatrix2D,
// src/BarycentricMatrix.jl:208-218, r <= 32).
struct HierBlock {
    int kind;
    int64_t row0, rows, col0, cols, rank;
    const double *data;
};

// Builds the flat plan and the host stores (panels, V, F) in FP64:
// low-rank blocks become coefficient slots whose basis panel is V diag(sigma)
// (read back by TCOEF pieces), core blocks slots whose far-field stage applies
// C, and rows are cut into the elementary intervals of all block row ranges.
int build_hier_plan(int64_t m, int64_t n, const std::vector<HierBlock> &blocks, Plan &P,
                    std::vector<double> &vstore, std::vector<double> &fstore, std::vector<double> &pstore);

// Merges independent plans into one block-diagonal plan: instance i's rows
// and columns follow those of instances 0..i-1, its slots, stores and records
// are offset accordingly, and the transfer bands are merged launch by launch
// (the k-th band launch of every instance runs together).
void merge_plans(const std::vector<Plan> &parts, Plan &out);

}  // namespace hm
