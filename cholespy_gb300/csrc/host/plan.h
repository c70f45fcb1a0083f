// Solve plan of a factor: the split of L into a row-wise leaf region and a
// supernodal top region, with the dense panel layout and the work units of
// the supernodal sweeps. Built on the host once per factor.
#pragma once
#include <cstdint>
#include <vector>

#include "host.h"

namespace gbchol {

constexpr int kChunk = 32;  // columns per supernodal work unit (one warp lane per row)

#ifdef __CUDACC__
#define GBCHOL_HD __host__ __device__
#else
#define GBCHOL_HD
#endif

// One dense block L[rows, cols of a source chunk] applied to a unit in the
// lower sweep: t[row - c0] -= L_block * x_src.
struct SnContrib {
    int64_t panel_off;  // element offset of the block's first (row, col) in the panel array
    int64_t rows_off;   // offset into sn_rows of the block's first row index
    int32_t ld;         // leading dimension of the source panel
    int32_t xcol;       // first column (permuted index) of the source chunk
    int32_t nr;         // rows of the block (<= kChunk)
    int32_t w;          // columns of the block (<= kChunk)
    int32_t src_unit;   // unit producing x_src
    uint32_t rowmask;   // bit p: the block has a row at unit row c0 + p (its
                        // i-th row is the i-th set bit: rows are sorted)
};

// A chunk of <= kChunk consecutive columns of one top-region supernode.
struct SnUnit {
    int32_t c0, w;          // columns [c0, c0 + w)
    int32_t ld;             // rows of the supernode's panel (its columns + off-diagonal rows)
    int32_t pos0;           // position of column c0 in the supernode's row list
    int64_t panel_col_off;  // element offset of column c0 (row position 0) in the panel array
    int64_t rows_off;       // offset of the supernode's row list in sn_rows
    int32_t contrib_begin;  // lower-sweep contributions the unit applies itself [begin, end)
    int32_t contrib_end;
    int32_t part_begin;     // lower-sweep partial sums the unit adds [begin, end)
    int32_t sn_w;           // width of the unit's supernode
    int32_t part_end;
    int32_t pad;
};

// A lower-sweep partial sum: the contributions [contrib_begin, contrib_end)
// of one unit's list, summed by a separate work item into a 32-row buffer
// slot. A unit hit by hundreds of source chunks (the chunks of a large
// separator) would otherwise apply them all in one CTA, serially with its
// dependency chain; its partial sums are ready as soon as their sources are.
struct SnPartial {
    int32_t unit;
    int32_t contrib_begin, contrib_end;
    int32_t pad;
};

struct SolvePlan {
    int32_t n = 0;
    // supernodes (fundamental) and the top-region marking
    std::vector<int32_t> sn_start;
    std::vector<char> sn_top;
    std::vector<char> row_top;            // column/row in the top region
    int32_t n_top_rows = 0;
    // top region: panels, row lists, units, contributions
    std::vector<int32_t> sn_rows;         // concatenated row lists of top supernodes
    std::vector<double> panels;           // column-major panels (FP64; cast for FP32)
    std::vector<SnUnit> units;            // in lower topological order
    std::vector<SnContrib> contribs;
    std::vector<SnPartial> parts;         // lower-sweep partial sums (by unit)
    std::vector<double> dinv;             // per unit: Dinv, M_lo, M_up (32x32 column-major each, plan.cpp)
    std::vector<double> fold2;            // per unit: M2_lo, M2_up (32x32 column-major each, plan.cpp)
    std::vector<int32_t> unit_order_lo;   // lower-sweep items in ticket order (sorted by key):
                                          // unit u (>= 0) or partial sum p (~p)
    std::vector<int32_t> unit_order_up;   // units in upper-sweep ticket order
    // ticket-order keys (estimated start, ns; larger than the key of every
    // item waited on): per unit, and per partial sum of the lower sweep
    std::vector<int32_t> unit_level_lo, unit_level_up;
    std::vector<int32_t> part_level_lo;
    std::vector<int32_t> unit_of_row;     // top rows: the unit holding the row (-1: leaf row)
    // leaf region, lower sweep: CSR over all rows. Leaf rows hold their full
    // row of L (diagonal last); top rows hold only their leaf-column entries.
    std::vector<int32_t> lo_rowptr, lo_cols;
    std::vector<double> lo_vals;
    std::vector<int32_t> lo_tasks;        // leaf rows in level order, then ~row for top rows
    std::vector<int32_t> lo_task_key;     // dependency level of each lower task (for merging)
    std::vector<int32_t> up_tasks;        // leaf rows by depth below the top region
    std::vector<int32_t> up_task_key;     // that depth, per task
    // upper sweep, leaf rows: columns of L split into the top-row part
    // (final before the leaf sweep starts: one wait-free "partial" pass) and
    // the diagonal + leaf-row part (the chained row sweep)
    std::vector<int32_t> upt_rowptr, upt_cols, upt_tasks;
    std::vector<double> upt_vals;
    std::vector<int32_t> upl_rowptr, upl_cols;
    std::vector<double> upl_vals;
    int32_t max_row_len = 0;
};

struct PlanOptions {
    int32_t min_top_width = 8;  // supernodes at least this wide (and their ancestors) are top
    // units with more than part_keep + part_group contribution blocks keep
    // their last part_keep blocks and hand the others to partial sums of
    // about part_group blocks each (0: no partial sums, the default: with
    // the estimated-start ticket order and the folded chain step, partial
    // sums measured slower on every RHS count)
    int32_t part_keep = 16;
    int32_t part_group = 0;
    // Ticket order of the leaf sweeps: a wavefront over groups of
    // leaf_group_rows consecutive rows (subtrees of the nested-dissection
    // order are row ranges), group g keyed leaf_skew levels after group g - 1
    // (the upper sweep from the last group down), so the x values a leaf row
    // gathers were written a few levels earlier by its own group and are
    // still in L2. Dependencies never point to a later group (lower sweep) /
    // an earlier one (upper sweep), so the order stays topological. 0 in
    // either: plain level order, the default: one system's leaf sweeps are
    // bound by their dependency chains, which the wavefront lengthens
    // (GB300, FP32, 64^3 / 128 RHS: 4.33 ms per solve in level order, 4.37 /
    // 4.56 / 5.11 ms with 32768 / 16384 / 8192 rows per group and skew 4;
    // icosphere 7 / 3 RHS: 0.94 -> 1.02 / 1.15 / 1.43 ms). The batch, whose
    // leaf sweeps are bound by their gathers, uses a wavefront over groups
    // of systems instead (batch.cu).
    int32_t leaf_group_rows = 0;
    int32_t leaf_skew = 0;
    // lower leaf sweep: the top rows' partial tasks after every leaf row
    // (true, the default) or each one past its own highest leaf input (false:
    // measured no faster, GB300 FP32: 64^3 / 128 RHS 4.22 vs 4.17 ms,
    // icosphere 7 / 3 RHS 0.853 vs 0.854 ms)
    bool partial_last = true;
};

// Upper-sweep blocks of the bulk supernodal sweeps, per unit in the order
// the unit applies them (the supernode's off-diagonal 32-row blocks, highest
// rows first, then its later chunks but the next, last first): where each
// block lies in the panels, which work-array rows it multiplies and which
// unit it waits for.
// Second folded block of the bulk sweeps: the unit's block from the chunk
// two before it (lower sweep) or two after it (upper sweep) in its own
// supernode, the last block of the unit's list, applied with the tile
// E L_block after the diagonal solve's product (x = E t' - M2 x_2 - M x_chain).
GBCHOL_HD inline bool snb_fold2_lo(const SnUnit& U) { return U.pos0 >= 2 * kChunk; }
GBCHOL_HD inline bool snb_fold2_up(const SnUnit& U) { return U.pos0 + U.w + kChunk < U.sn_w; }

struct SnbUpperPlan {
    std::vector<int32_t> begin;  // per unit: first block (n_units + 1 entries)
    std::vector<int64_t> src;    // panel offset of (block row 0, unit column 0)
    std::vector<int32_t> ld;     // leading dimension of that panel
    std::vector<int32_t> nrw;    // block rows | unit columns << 16
    std::vector<int32_t> dep;    // unit whose flag the block waits for
    std::vector<int32_t> rows;   // 32 per block: permuted row of each block row, -1 past the block
};

void build_snb_upper(const SolvePlan& P, SnbUpperPlan& U);

// Lower-sweep work of the bulk supernodal sweeps and the ticket order of
// both bulk sweeps. A unit's contribution list (without the chain block) is
// cut into groups: consecutive blocks from consecutive chunks of one other
// supernode (same rows of the unit, contiguous source columns and L tiles)
// form one group of up to max_cols source columns, applied as one block and
// waiting only for the flag of its last chunk (the chunks of a supernode
// finish in order); blocks from earlier chunks of the unit's own supernode
// stay single. A unit with more than keep + group groups applies only its
// last `keep` groups itself; the earlier ones go to partial sums of about
// `group` groups (separate items, started as soon as their sources are done)
// that the unit adds in a fixed order. Ticket keys come from the start-time
// estimate of build_plan with costs for one item applying its groups one
// after the other (blk_ns each).
struct SnbGroup {
    int32_t first;     // first contribution block (its L tile starts the group's tile rows)
    int32_t cols;      // source columns (tile rows) of the group
    int32_t src_unit;  // unit of the group's last chunk
    int32_t xcol;      // first source column
    uint32_t rowmask;  // the unit rows the group has
};

struct SnbOptions {
    int32_t keep = 16;
    int32_t group = 0;        // 0: no partial sums
    int32_t max_cols = 64;    // source columns per group (32: no merging)
    bool order_by_finish = true;  // a unit's groups in estimated source-finish order (else source order)
    int64_t lat_ns = 1000;    // flag latency
    int64_t base_ns = 5000;   // fixed cost of an item (diagonal solve, chain step)
    // cost of one block. Measured at 64^3, 128 RHS (5.99 / 5.87 / 5.79 /
    // 5.73 / 5.75 ms per solve for 2.5 / 4 / 6 / 9 / 15 us): a long list is
    // best started as soon as its first source is done, ahead of the estimate.
    int64_t blk_ns = 9000;
    // 2: the block of the chunk before the chain one is a group of its own,
    // the unit's last (the sweeps may then fold it: snb_fold2_lo); 1: it is
    // ordered like the others.
    int32_t fold = 2;
};

struct SnbLowerPlan {
    std::vector<SnbGroup> groups;     // per unit in list order (chain block excluded)
    std::vector<int32_t> unit_info;   // per unit: first group it applies itself, end of its groups,
                                      // first and end partial sum
    std::vector<SnPartial> parts;     // partial sums over group ranges (contrib_begin/end = groups)
    std::vector<int32_t> order_lo;    // lower-sweep tickets: unit u, or partial p as ~p
    std::vector<int32_t> order_up;    // upper-sweep tickets: units
};

void build_snb_lower(const SolvePlan& P, const SnbUpperPlan& B, const SnbOptions& o, SnbLowerPlan& L);

// Builds the plan from a factor and the level orders of L and L^T (rows
// sorted by (level, row)).
void build_plan(const Factor& F, const std::vector<int32_t>& lower_order,
                const std::vector<int32_t>& upper_order, const PlanOptions& opt, SolvePlan& P);

}  // namespace gbchol
