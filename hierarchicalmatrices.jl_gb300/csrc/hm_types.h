// Device-table records shared by the host planner and the CUDA kernels.
//
// A KernelMatrix (src/KernelMatrix.jl:47-116) is flattened into:
//   * coefficient "slots": one per node of the row (x) and column (y) cluster
//     trees that carries Chebyshev coefficients, each `width` values per
//     right-hand side;
//   * V panels: explicit column-cluster bases (y side) whose transpose times
//     x gives the coefficients of a leaf slot;
//   * transfer steps: parent <- children moves of coefficients between tree
//     levels (upward on the column tree, downward on the row tree);
//   * M2L rows: for each row cluster, the barycentric blocks
//     (src/BarycentricMatrix.jl:208-297) of that row, each an r x r sample
//     matrix F applied to the coefficients of its column cluster;
//   * row segments: a contiguous run of rows whose near-field dense blocks and
//     row basis are the same, stored as one column-major panel
//     [U rows | dense block rows ...] that multiplies a gathered right-hand
//     side [s coefficients ; x segments ...].
#pragma once
#include <stdint.h>

struct hm_vpanel {      // explicit basis panel: coef[slot][col0 + m] = (P^T x[row0 : row0+nrows))[m]
    int64_t row0;       // first row of x (element index before stride)
    int64_t off;        // element offset of the panel in the V store
    int32_t nrows;
    int32_t ld;         // row stride of the row-major panel
    int32_t width;      // number of basis columns (<= 32)
    int32_t slot;
    int32_t col0;       // first coefficient of the slot this panel produces
    int32_t pad;
};

struct hm_xfer {        // coefficient transfer between a node and its two children
    int32_t slot, c0, c1, pad;
};

// Transfer bands: the upward (downward) transfers are grouped into bands of a
// few tree levels; a band is one launch, each of its tasks (a subtree cut to
// the band's levels) one CTA, which walks the task's steps (one level each)
// in order with a CTA barrier between steps.
struct hm_task { int32_t step0, step1; };     // range of steps
struct hm_step { int32_t e0, e1; };           // range of transfer records

struct hm_m2l_row {     // s[slot] = sum_{e in [begin,end)} F_e t[yslot_e]
    int32_t slot, begin, end, pad;
};

struct hm_m2l_ent {
    int64_t foff;       // element offset of F_e (r x r column-major)
    int32_t yslot, pad;
};

struct hm_seg {         // y[row0 : row0+nrows) (+)= panel * gathered rhs
    int64_t row0;
    int64_t poff;       // element offset of the panel in the panel store
    int32_t nrows;
    int32_t ld;
    int32_t width;      // total panel columns
    int32_t piece0;     // first piece record
    int32_t npieces;
    int32_t nfar;       // far-field columns: the pieces other than X come first
};

enum {
    HM_PIECE_COEF = 0,   // far-field coefficients s[slot] (after the far-field stage)
    HM_PIECE_X = 1,      // a run of x
    HM_PIECE_TCOEF = 2   // coefficients t[slot] straight from a basis panel (low-rank blocks)
};

struct hm_piece {       // one block column run of a segment panel
    int64_t src;        // coefficient slot (COEF) or first x element (X)
    int32_t kind;
    int32_t width;
};
static_assert(sizeof(hm_seg) == 40 && sizeof(hm_piece) == 16, "records are copied as 8-byte words");

// Build-time only: geometry needed to fill factors on the device.
struct hm_fill_vpanel { double a, b; };          // box of an explicit basis panel
struct hm_fill_f { double xa, xb, ya, yb; };     // boxes of one F block
struct hm_fill_seg {                              // what the panel columns hold
    double a, b;        // row-basis box (when has_basis)
    int32_t has_basis;  // first `basis_w` columns are the row basis
    int32_t basis_w;
};
