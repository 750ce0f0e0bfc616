// pf_internal.h - device data layout and kernel launchers of the fill pipeline.
#pragma once

#include <cuda_bf16.h>
#include <cuda_runtime.h>
#include <stdint.h>

#include "pfcuda.h"

namespace pfc {

constexpr int kTile = 16;
// Coverage is accumulated as int32 fixed point with this many fraction bits:
// integer sums do not depend on the order fills are visited in.
constexpr int kCovShift = 20;
constexpr int kMaxDepth = 32;              // flattening recursion bound (depth of the d3d9 bisection)
constexpr uint32_t kMaxWalk = 1u << 20;    // tile-walk step bound per line
constexpr uint32_t kNone = 0xffffffffu;       // also the scene format's "no clip path"
constexpr uint32_t kPathIsClip = 8u;           // PathDev::flags: a clip path (tiled, never drawn)

// Learned sizer: per-path features -> 64 -> 64 -> (log1p leaf lines, log1p fills).
constexpr int kSizerIn = 12, kSizerHidden = 64, kSizerOut = 2;
constexpr int kSizerParams = kSizerHidden * kSizerIn + kSizerHidden + kSizerHidden * kSizerHidden + kSizerHidden +
                             kSizerOut * kSizerHidden + kSizerOut;  // 5122

// Kernel error bits (written with atomicOr into the status word).
enum : uint32_t {
    kErrDepth = 1u << 0,    // flattening hit kMaxDepth
    kErrWalk = 1u << 1,     // a tile walk hit kMaxWalk
    kErrClip = 1u << 2,     // Cohen-Sutherland clipping did not settle
    kErrNonFinite = 1u << 3,// a point is NaN or infinite
    kErrScanWait = 1u << 4, // a scan's look-back wait hit its bound
    kErrStroke = 1u << 5,   // a dash pattern ran past its step bound or a cap search past its ring
    kErrOverflowSeg = 1u << 8,
    kErrOverflowLeaf = 1u << 9,
    kErrOverflowFill = 1u << 10,
    kErrOverflowList = 1u << 11,
};

// Per scene of a batch (device).
struct SceneDev {
    float vb_left, vb_top;  // view box (Scene::set_view_box): tiling clips against it
    float vb_right;       // view box right edge, rounded up to a multiple of 16
    float vb_bottom;      // view box bottom edge
    uint32_t fbw, fbh;    // framebuffer tiles across / down
    uint32_t fb_first;    // first framebuffer tile of this scene in the batch
    uint32_t img_w, img_h;
    uint32_t clear;       // RGBA8
    uint64_t img_offset;  // byte offset of the scene's image in the batch image buffer
    uint32_t path_first, path_end;
    uint32_t contour_first, contour_end;
    uint32_t point_first, point_end;
    uint32_t cstart_base, pstart_base;  // offsets of the scene's offset arrays
    uint32_t row_first;                  // first framebuffer-tile row of this scene in the batch
    uint32_t load;                       // PF_LOAD_LOAD: composite over the image already there
};

// Per draw path (device), written by the set-up kernel.
struct PathDev {
    int32_t rx0, ry0, rx1, ry1;  // tile rect (BuiltPath::tile_bounds)
    uint32_t tile_first;         // first global tile
    uint32_t col_first;          // first global column
    uint32_t scene;
    uint32_t flags;              // bit0 even-odd, bit1 occludes (opaque src-over), bit3 clip path
};

// Segment record: points index a, kind, and the second point for closing lines.
enum : uint32_t { kSegLine = 0, kSegQuad = 1, kSegCubic = 2, kSegClose = 3 };
struct SegDev {
    uint32_t a;       // first point (global)
    uint32_t b;       // kSegClose: the contour's first point; else unused
    uint32_t kind;
    uint32_t path;
};

// Everything the kernels read and write for one batch.
struct Batch {
    // inputs (concatenated per-scene arrays)
    const float2 *points;
    const uint8_t *flags;
    const uint32_t *contour_start_cat;   // per scene n_contours+1 entries, scene-local
    const uint32_t *path_start_cat;      // per scene n_paths+1 entries, scene-local
    const uint8_t *fill_rule;
    const uint32_t *color;
    const uint32_t *path_clip_cat;       // per uploaded path: scene-local clip path, kNone (or null:
                                         // no clip paths in the batch)
    const uint8_t *path_is_clip_cat;     // per uploaded path: 1 for a clip path
    uint32_t *path_clip_rel;             // [n_paths] the clip path within the frame, kNone
    const uint32_t *path_grad;           // per uploaded path: its gradient, kNone (or null: no
                                         // gradients in the batch)
    const float4 *grad_meta;             // [gradients][4]: the shader's half-float metadata (3 x 4
                                         // floats) and (type, wrap, opaque, -) as bits
    const uint32_t *grad_ramp;           // [gradients][256] RGBA8 ramps
    const SceneDev *scenes;
    const uint32_t *scene_path_first;    // [n_scenes_all + 1]
    const uint32_t *scene_contour_first; // [n_scenes_all + 1]
    const uint32_t *scene_fb_first;      // [n_scenes_all + 1]
    const uint32_t *fb_scene;            // [framebuffer tiles of all scenes] the scene of each
    const uint32_t *scene_row_first;     // [n_scenes_all + 1]
    uint32_t n_scenes_all;               // scenes uploaded
    // the scenes rendered by this frame: a contiguous range of the uploaded ones.
    // Per-frame arrays are indexed from 0 = the range's first path / contour / framebuffer tile.
    uint32_t scene_base, n_scenes;
    uint32_t path_base, n_paths;
    uint32_t contour_base, n_contours;
    uint32_t fb_base, row_base;

    // normalised topology
    uint32_t *contour_point_first;       // [n_contours + 1] global
    uint32_t *contour_path;              // [n_contours]
    PathDev *paths;                      // [n_paths]
    float4 *path_bounds;                 // [n_paths] outline bounds (min x, min y, max x, max y)
    // learned frame: per-path leaf regions laid out from the sizer's budgets
    uint32_t *path_leaf_first;           // [n_paths + 1] budgets -> scanned
    uint32_t *path_leaf_budget;          // [n_paths]
    uint32_t *path_leaf_cursor;          // [n_paths]
    uint32_t leaf_pool_first, leaf_pool_cap;  // shared spill pool after the per-path regions
    // per-path binning: leaf range of every path, paths bucketed by tile count
    uint2 *path_leaf_range;              // [n_paths] [first, end) in the leaf buffer
    const uint2 *path_contours;          // [n_paths] [first, end) contours of each path
    uint32_t *bin_list;                  // [4][n_paths] paths of each size class
    uint32_t *bin_ctl;                   // [16] class counts, work tickets
    uint32_t *path_tiles;                // [n_paths + 1] -> scanned to first tile
    uint32_t *path_cols;                 // [n_paths + 1] -> scanned to first column
    uint32_t *contour_segs;              // [n_contours + 1] -> scanned

    // segments / leaves
    SegDev *segs;
    uint32_t seg_cap;
    uint32_t *seg_order;                 // [segs] the order the flattening kernels take them in
    uint32_t *seg_leaves;                // [segs + 1] -> scanned
    float4 *leaves;
    uint32_t leaf_cap;
    // learned frame: the spill pool's lines listed by path.  pool_cnt points one past the start
    // of its allocation (pool_cnt[-1] == 0); once listed, path p's pooled lines are
    // pool_idx[pool_cnt[p - 1] .. pool_cnt[p]).  Null in an exact frame.
    uint32_t *pool_path;                 // [pool cap] path of each pooled line
    uint32_t *pool_cnt;                  // [-1 .. n_paths]
    uint32_t *pool_idx;                  // [pool cap]

    // tiles.  Each path's fills are one block starting at path_fill[p], grouped by tile in the
    // path's row-major tile order; tile_fills[t] is one past the last fill of tile t, so the
    // fills of tile t are [t == the path's first tile ? path_fill[p] : tile_fills[t - 1],
    // tile_fills[t]).  (Class-3 paths use tile_fills as counters, then cursors, on the way.)
    uint32_t *tile_fills;                // [tiles]
    uint32_t *path_fill;                 // [n_paths] first fill of each path
    uint8_t *path_cls;                   // [n_paths] binning class (0xff: no columns)
    uint16_t *tile_state;                // [tiles] propagated int8 backdrop | alpha << 8
    int32_t *col_above;                  // [cols] deltas landing above the rect
    int32_t *col_final;                  // [cols]
    uint2 *fills;                        // [fills] packed u16 x4
    uint32_t fill_cap;
    uint2 *stage;                        // per binning CTA: fills staged during its count walk

    // per framebuffer-tile row of each scene: the paths whose tile rect spans the row,
    // in path order
    uint32_t *row_first;                 // [rows + 1] counts -> scanned
    uint4 *row_paths;                    // {path, rx0 | rx1 << 16, tile of (0, row) in the path's rect
                                         //  numbering, path flags}
    uint32_t row_cap;
    uint32_t n_rows;
    uint32_t n_fb;

    // composite-list dump (canonical output only)
    int32_t *z;                          // [fb tiles]
    uint32_t *fb_count;                  // [fb + 1] -> scanned
    uint32_t *list;

    uint8_t *image;                      // batch image buffer
    uint32_t *status;                    // [kStCount] error bits and totals
    uint32_t counters;                   // nonzero: the composite adds its work counters to status
    // launch parameters (pf_tuning): lines spanning more tiles than long_line are walked by a
    // whole warp; comp_ticket > 0: the composite's warps stay resident and take that many
    // framebuffer tiles per ticket (0: one warp per tile)
    float long_line;
    uint32_t comp_ticket;
};

// The launch parameters of a frame (pf_tuning), as the kernels and launchers read them.
struct Tuning {
    uint32_t bin_ctas_per_sm[3] = {0, 0, 0};  // 0: as many as fit
    float long_line = 8.0f;
    bool bin_concurrent = false;
    bool seg_sorted = true;
    uint32_t comp_ticket = 0;
};

// status word slots: error bits, then the totals the scans produce
enum : int {
    kStErr = 0,
    kStSegs = 1,
    kStTiles = 2,
    kStCols = 3,
    kStLeaves = 4,
    kStAlphaTiles = 5, // frame counters: alpha tiles of the draw paths
    kStList = 6,
    kStListFills = 7,  // fills of the alpha tiles that made it into composite lists
    kStRows = 8,       // entries of the per-row path lists
    kStEntries = 9,    // composite entries (visible tiles at or above the occluder)
    kStLeafBudget = 10,// learned frame: sum of per-path leaf budgets
    kStFillBudget = 11,// learned frame: sum of per-path fill estimates
    kStLeafCount = 12, // learned frame: leaf lines produced (kept or not)
    kStPoolUsed = 13,  // learned frame: leaf slots taken from the spill pool
    kStPathsOver = 14, // learned frame: paths that overran their leaf budget
    kStWalkChunks = 15,// composite: 32-candidate chunks walked (all framebuffer tiles)
    kStFill64 = 16,    // two words: fills reserved by the frame's paths (64-bit)
    kStPoolListed = 18,// learned frame: pooled lines listed by path
    kStVisible = 19,   // frame counters: visible tiles of the draw paths (alpha, or a nonzero backdrop)
    kStFlatTicket = 20,// learned frame: groups of 32 segments taken by the flattening warps
    kStCount = 21,
};

// Kernels launched by this library (host-side counter, all contexts).
uint64_t launches();
void count_launches(uint32_t n);

// Scans (exclusive, in place allowed); the total lands in *total (device).
size_t scan_temp_bytes(uint32_t n);
cudaError_t scan_exclusive_u32(const uint32_t *in, uint32_t *out, uint32_t n, uint32_t *total, void *temp,
                               cudaStream_t st, uint32_t *err);

// Stroke-to-fill and dashing at upload (pf_stroke.cu).  Inputs: the uploaded outline in the
// upload's per-scene layout; outputs: the dashed contours, one job per output contour, and the
// new outline.
struct StrokeIn {
    uint32_t n_paths, n_scenes, n_jobs, n_out_points;
    const SceneDev *scenes;             // the input layout's scene table
    const uint32_t *scene_path_first;   // [n_scenes + 1]
    const uint32_t *scene_contour_first;
    const uint32_t *cstart, *pstart;    // scene-local offset arrays
    const float2 *points;
    const uint8_t *flags;
    const uint8_t *closed;              // [contours] or null
    const pf_stroke *stroke;            // [n_paths] (dash_first rebased into dashes)
    const float *dashes;
    uint32_t *dash_pts, *dash_cnt;      // [n_paths + 1] counts -> scanned
    uint32_t *dash_end;                 // [dash contours] one past each contour's last point
    float2 *dash_points;
    uint8_t *dash_flags;
    uint32_t *job_first;                // [n_paths + 1] counts -> scanned
    uint4 *jobs;                        // [n_jobs]
    uint32_t *job_pts;                  // [n_jobs + 1] counts -> scanned
    float2 *out_points;
    uint8_t *out_flags;
    // the segment-parallel stroker: one unit per input segment and direction, one leaf per
    // offset piece; a job whose contour is degenerate is redone by the sequential kernel
    uint32_t n_units, n_leaves;
    uint32_t *job_units;                // [n_jobs + 1] counts -> scanned
    uint32_t *job_nfwd;                 // [n_jobs] units of the forward direction
    uint32_t *job_flags;                // [n_jobs] bit 0: done by the sequential kernel
    uint32_t *job_cap1, *job_end;       // [n_jobs] points of the first cap / of the end (cap, join)
    float4 *units;                      // [n_units][3] segment, (job, direction | index)
    uint32_t *unit_leaves;              // [n_units + 1] counts -> scanned
    float4 *leaves;                     // [n_leaves][3] piece, join point, (job, meta)
    uint32_t *leaf_pts;                 // [n_leaves + 1] counts -> scanned
    const uint32_t *unit_order;         // [n_units] units, the most work first (or null)
    const uint32_t *dash_order;         // [n_dashed] the dashed paths, the most work first
    uint32_t n_dashed;
};
size_t stroke_order_ctl_bytes();
cudaError_t launch_stroke_order(const StrokeIn &in, int what, uint32_t *ctl, uint32_t *order, cudaStream_t st);
cudaError_t launch_dash(const StrokeIn &in, bool write, uint32_t *status, cudaStream_t st);
cudaError_t launch_copy_words(uint32_t *dst, const uint32_t *src, uint32_t n, cudaStream_t st);
// up to 8 single words gathered into dst[0, n)
struct WordSources {
    const uint32_t *p[8];
    uint32_t n;
};
cudaError_t launch_gather_words(uint32_t *dst, const WordSources &s, cudaStream_t st);
cudaError_t launch_copy_bytes(uint8_t *dst, const uint8_t *src, uint32_t n, cudaStream_t st);
cudaError_t launch_stroke_jobs(const StrokeIn &in, bool fill, cudaStream_t st);
cudaError_t launch_stroke(const StrokeIn &in, bool write, uint32_t *status, cudaStream_t st);
cudaError_t launch_units(const StrokeIn &in, bool write, cudaStream_t st);
cudaError_t launch_unit_leaves(const StrokeIn &in, bool write, cudaStream_t st);
cudaError_t launch_job_ends(const StrokeIn &in, bool write, cudaStream_t st);
cudaError_t launch_leaf_pts(const StrokeIn &in, bool write, cudaStream_t st);
cudaError_t launch_job_totals(const StrokeIn &in, uint32_t *status, cudaStream_t st);
cudaError_t launch_outline_starts(const StrokeIn &in, const SceneDev *out_scenes, uint32_t *cstart,
                                  uint32_t *pstart, cudaStream_t st);
cudaError_t launch_scene_bounds(const StrokeIn &in, uint32_t *out, cudaStream_t st);

// Gradient paints at upload (pf_paint.cu).  paints: every uploaded path's pf_paint; stops: every
// scene's stops, scene s's from stop_base[s].  launch_gradient_index numbers the gradient paths
// (path_grad[p], kNone for solid ones; grad_path[g]); launch_gradients orders each gradient's
// stops as Gradient::add does and builds its ramp and shader metadata.
constexpr uint32_t kMaxGradientStops = 1024;
cudaError_t launch_gradient_index(const pf_paint *paints, uint32_t n_paths, uint32_t *flags, uint32_t *path_grad,
                                  uint32_t *grad_path, void *scan_temp, uint32_t *status, cudaStream_t st);
cudaError_t launch_gradients(const pf_paint *paints, const uint32_t *grad_path, const uint32_t *scene_path_first,
                             uint32_t n_scenes, const uint32_t *stop_base, const pf_color_stop *stops, uint32_t n,
                             float4 *meta, uint32_t *ramps, cudaStream_t st);

// Stage launchers (all asynchronous on the given stream).
cudaError_t launch_normalize(const Batch &b, uint2 *path_contours, cudaStream_t st);
cudaError_t launch_path_setup(const Batch &b, const uint2 *path_contours, cudaStream_t st);
cudaError_t launch_path_offsets(const Batch &b, cudaStream_t st);
cudaError_t launch_contour_segments(const Batch &b, bool write, cudaStream_t st);
cudaError_t launch_flatten(const Batch &b, uint32_t n_segs, bool write, cudaStream_t st, uint64_t n_lines = 0);
cudaError_t launch_rows(const Batch &b, bool write, cudaStream_t st);
cudaError_t launch_composite(const Batch &b, cudaStream_t st);  // b.comp_ticket picks the grid
// fb_scene[t] = the scene of framebuffer tile t, for every uploaded scene (at upload).
cudaError_t launch_fb_scene(const uint32_t *scene_fb_first, uint32_t n_scenes, uint32_t *fb_scene, cudaStream_t st);
// Frame counters: alpha and visible tiles of the draw paths into the status words.
cudaError_t launch_tile_counts(const Batch &b, cudaStream_t st);
cudaError_t launch_list_dump(const Batch &b, bool write, cudaStream_t st);
// Canonical output of clipped frames: every tile's state after the clip rules and its clip tile.
cudaError_t launch_clip_dump(const Batch &b, uint32_t n_tiles, uint32_t *state, uint32_t *clip, cudaStream_t st);
cudaError_t launch_coverage_dump(const Batch &b, const uint32_t *tiles, uint32_t n, float *out, cudaStream_t st);

// Learned sizer (pf_sizer.cu).
cudaError_t launch_features(const Batch &b, const uint2 *path_contours, float4 *contour_scratch, float *feat,
                            cudaStream_t st);
cudaError_t launch_budgets(const Batch &b, const float *pred, float mul, float add, uint32_t *leaf_budget,
                           uint32_t *fill_budget, uint32_t *leaf_cursor, cudaStream_t st);
cudaError_t launch_path_counts(const Batch &b, const uint2 *path_contours, uint32_t *leaves, uint32_t *fills,
                               cudaStream_t st);
cudaError_t launch_flatten_budget(const Batch &b, uint32_t n_segs, cudaStream_t st);
// Orders the segments by estimated subdivision depth (seg_order); ctl holds 32 words.
cudaError_t launch_seg_order(const Batch &b, uint32_t n_segs, uint32_t *ctl, cudaStream_t st);
size_t seg_ctl_bytes();  // the per-block bucket counts launch_seg_order keeps in ctl
// Binning by path: classify (leaf ranges, size classes), then bin every path (counts,
// backdrops, fill offsets, fills).  A learned frame first lists its pooled lines by path:
// count, scan pool_cnt, scatter.
cudaError_t launch_bin_classify(const Batch &b, bool learned, cudaStream_t st);
// side[0..1], fork, join[0..1]: streams and events for running the CTA classes concurrently
// (tuning.bin_concurrent), or null.
struct BinStreams {
    cudaStream_t side[2];
    cudaEvent_t fork, join[2];
};
cudaError_t launch_bin_paths(const Batch &b, const Tuning &t, const BinStreams *bs, cudaStream_t st);
// The most CTAs of each binning class one SM holds.
cudaError_t bin_class_max_ctas(int out[3]);
cudaError_t launch_pool_lists(const Batch &b, bool scatter, cudaStream_t st);
// Bytes of the binning CTAs' fill stage on the current device for these launch parameters.
cudaError_t bin_stage_bytes(const Tuning &t, size_t *bytes);
cudaError_t launch_mlp_predict(const __nv_bfloat16 *w, const float *feat, uint32_t n, float *out, cudaStream_t st);
cudaError_t launch_mlp_grad(const __nv_bfloat16 *w, const float *feat, const float *target, const uint32_t *index,
                            uint32_t n, float *grad, float *loss, cudaStream_t st);
cudaError_t launch_adam(float *master, __nv_bfloat16 *w, float *grad, float *m, float *v, float lr, int step,
                        cudaStream_t st);

}  // namespace pfc
