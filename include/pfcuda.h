/*
 * pfcuda.h - C-ABI of the GB300 (sm_103a) GPU-driven fill pipeline.
 *
 * The pipeline replaces the stages of pathfinder-cpp's GpuDriven renderer
 * (RendererD3D11::draw, pathfinder/core/d3d11/renderer.cpp:302-336, and the
 * compute shaders pathfinder/shaders/d3d11/{bound,dice,bin,propagate,sort,
 * fill,tile}.comp) with hand-written CUDA kernels, and computes the integer
 * tile data with the semantics of the reference's CPU tiler
 * (pathfinder/core/d3d9/tiler.cpp, object_builder.cpp, scene_builder.cpp).
 *
 * Conventions
 *  - Every entry point returns an int status: PF_OK (0) or a pf_status > 0.
 *    Nothing aborts; the last error text of a context is pf_last_error().
 *  - Host arrays passed in are borrowed for the duration of the call only.
 *  - Device memory is owned by the context.  One context per host thread;
 *    calls on one context are serialised by the caller.
 *  - A context works on the CUDA stream given in pf_config (0 = a stream the
 *    context creates).  Entry points return once their work is queued unless
 *    they hand results back to host memory, in which case they synchronise.
 */
#ifndef PFCUDA_H
#define PFCUDA_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define PF_ABI_VERSION 5

typedef enum pf_status {
    PF_OK = 0,
    PF_ERR_INVALID_ARGUMENT = 1, /* null pointer, bad size, malformed offsets */
    PF_ERR_CUDA = 2,             /* a CUDA runtime call failed                */
    PF_ERR_OUT_OF_MEMORY = 3,    /* device allocation failed                  */
    PF_ERR_OVERFLOW = 4,         /* a fixed capacity was exceeded             */
    PF_ERR_KERNEL_LIMIT = 5,     /* a kernel hit an iteration bound           */
    PF_ERR_NOT_READY = 6         /* no scene uploaded / nothing rendered yet  */
} pf_status;

/* Fill rules (pathfinder/core/data/data.h:136-141). */
#define PF_FILL_NONZERO 0u
#define PF_FILL_EVEN_ODD 1u

/* No clip path (pf_scene_view::path_clip). */
#define PF_NO_CLIP 0xffffffffu

/* Line caps and joins (LineCap, LineJoin, pathfinder/core/data/data.h:73-96). */
#define PF_CAP_BUTT 0u
#define PF_CAP_SQUARE 1u
#define PF_CAP_ROUND 2u
#define PF_JOIN_MITER 0u
#define PF_JOIN_BEVEL 1u
#define PF_JOIN_ROUND 2u

/*
 * How a path is stroked: StrokeStyle (pathfinder/core/stroke.h:14-27) and the canvas's line
 * dash (Canvas::stroke_path, pathfinder/core/canvas.cpp:270-300).  A stroked path's outline is
 * dashed (OutlineDash, pathfinder/core/dash.cpp) when it has a pattern, then converted to its
 * stroke outline (OutlineStrokeToFill, pathfinder/core/stroke.cpp) on the GPU when the scene is
 * uploaded; the stroke outline is filled with the nonzero rule, as the canvas does.
 */
typedef struct pf_stroke {
    float line_width;    /* > 0: the path is stroked with this width; 0: it is filled      */
    float miter_limit;   /* PF_JOIN_MITER: the miter limit ratio                            */
    uint8_t line_cap;    /* PF_CAP_*                                                       */
    uint8_t line_join;   /* PF_JOIN_*                                                      */
    uint16_t reserved;
    uint32_t dash_first; /* the dash pattern: dashes[dash_first, dash_first + dash_count) */
    uint32_t dash_count; /* 0: a solid stroke                                              */
    float dash_offset;   /* the pattern's phase (the canvas passes 0)                      */
} pf_stroke;

/*
 * Gradient paints (Paint::from_gradient, pathfinder/core/paint/paint.h:87-95; Gradient,
 * core/paint/gradient.h): the path is filled with a 256-texel colour ramp (GradientTileBuilder::
 * allocate, core/paint/gradient.cpp) sampled per pixel as tile.comp samples its colour texture:
 * linearly filtered, clamped or repeated along the ramp, with the metadata (the gradient's
 * texture transform and radial parameters) stored as half floats the way the reference's
 * RGBA16F metadata texture stores them (core/renderer.cpp:167-250).
 */
#define PF_PAINT_SOLID 0u   /* the path's colour */
#define PF_PAINT_LINEAR 1u  /* GradientLinear: t runs from line.from (0) to line.to (1) */
#define PF_PAINT_RADIAL 2u  /* GradientRadial: circles (from, r0) to (to, r1), then transform */
#define PF_WRAP_CLAMP 0u
#define PF_WRAP_REPEAT 1u

typedef struct pf_color_stop {
    float offset;    /* position along the gradient, [0, 1] */
    uint32_t color;  /* RGBA8, red in the low byte */
} pf_color_stop;

typedef struct pf_paint {
    uint32_t type;        /* PF_PAINT_*                                              */
    uint32_t wrap;        /* PF_WRAP_*                                               */
    uint32_t stop_first;  /* the colour stops, in the order Gradient::add_color_stop  */
    uint32_t stop_count;  /* receives them: stops[stop_first, stop_first + count)      */
    float line[4];        /* from.x, from.y, to.x, to.y                               */
    float radii[2];       /* PF_PAINT_RADIAL: r0, r1                                   */
    float transform[6];   /* PF_PAINT_RADIAL: m11, m21, m12, m22, m13, m23 (x' = m11 x +
                             m12 y + m13); the identity is {1, 0, 0, 1, 0, 0}            */
} pf_paint;

/* What a frame does with the destination image before it composites (the tile shader's load
 * actions, pathfinder/shaders/d3d11/tile.comp:9-10, 744-757; Renderer::draw's
 * clear_dst_texture, pathfinder/core/d3d11/renderer.cpp:376-380). */
#define PF_LOAD_CLEAR 0u /* every pixel starts as clear_color                                    */
#define PF_LOAD_LOAD 1u  /* every pixel starts as the image already there (the last frame's image,
                            or what pf_write_image put there)                                     */

/* Point flags (pathfinder/core/data/data.h:120-129). */
#define PF_POINT_ON_CURVE 0u
#define PF_POINT_CONTROL_0 1u
#define PF_POINT_CONTROL_1 2u

/*
 * One scene in outline form: the data the reference's Scene holds for its
 * draw paths (Scene::draw_paths -> DrawPath::outline -> Outline::contours,
 * pathfinder/core/scene.h, pathfinder/core/data/path.h:11-40,
 * pathfinder/core/data/contour.h:16-30).  Outlines are already transformed
 * into canvas space (Canvas::push_path, pathfinder/core/canvas.cpp:180-190).
 *
 *   points        [n_points][2] float32, x then y
 *   point_flags   [n_points]    PF_POINT_*
 *   contour_start [n_contours + 1]  offsets into points (non-decreasing)
 *   path_start    [n_paths + 1]     offsets into contours (non-decreasing)
 *   fill_rule     [n_paths]     PF_FILL_*
 *   color         [n_paths]     RGBA8 solid paint, red in the low byte;
 *                               src-over (pathfinder/shaders/d3d11/tile.comp:841)
 *   width,height  size of the destination image in pixels (ceil(width) x ceil(height)
 *                 RGBA8); framebuffer tiles cover it from (0, 0), as the tile shader's
 *                 dispatch covers the destination texture (renderer.cpp:371, 443)
 *   clear_color   RGBA8 colour the destination is cleared to
 *   path_clip     [n_paths] or NULL: the scene-local index of the clip path of each path, or
 *                 PF_NO_CLIP (DrawPath::clip_path, pathfinder/core/data/path.h:36)
 *   path_is_clip  [n_paths] or NULL: 1 for a clip path (Scene::clip_paths, ClipPath,
 *                 pathfinder/core/data/path.h:45-57): tiled like the others, never drawn, and
 *                 not clipped itself.  Clip paths follow all draw paths.  A clipped draw tile
 *                 follows Tiler::prepare_tiles (pathfinder/core/d3d9/tiler.cpp:386-431): culled
 *                 outside the clip's rect or over a blank clip tile, drawn with the clip's mask
 *                 when it is solid and the clip tile is an alpha tile, and drawn with the two
 *                 masks combined (tile_clip_combine.frag: min of |mask + backdrop|) when both
 *                 are alpha tiles.
 *   path_stroke   [n_paths] or NULL: how each path is stroked (line_width 0: filled)
 *   contour_closed [n_contours] or NULL (every contour open): Contour::closed
 *                 (pathfinder/core/data/contour.h:27), which decides between caps and a
 *                 closing join when the contour is stroked; fills close every contour
 *   dashes        [n_dashes]: the dash patterns the strokes refer to; finite, >= 0, and each
 *                 pattern's total > 0
 *   path_paint    [n_paths] or NULL (every path solid): each path's paint; a gradient path's
 *                 colour entry is ignored (its base colour is opaque white, as from_gradient's)
 *   stops         [n_stops]: the colour stops the gradients refer to
 *   view_box      [4] or NULL: the scene's view box (Scene::set_view_box,
 *                 pathfinder/core/scene.cpp:169-176) as left, top, right, bottom; NULL is
 *                 (0, 0, width, height).  Its right edge is rounded up to a multiple of 16 as
 *                 set_view_box does.  Path tile rects are the paths' bounds intersected with it
 *                 (core/d3d9/tiler.cpp:317-335) and lines are clipped to its left, right and
 *                 bottom edges (tiler.cpp:141-153); tiles keep canvas coordinates, so a tile
 *                 (x, y) lands on pixels [16x, 16x + 16) x [16y, 16y + 16) of the image, and a
 *                 tile outside the image is never composited.  Coordinates in [-65536, 65536],
 *                 left <= right, top <= bottom.
 *   load_action   PF_LOAD_CLEAR or PF_LOAD_LOAD
 */
typedef struct pf_scene_view {
    const float *points;
    const uint8_t *point_flags;
    const uint32_t *contour_start;
    const uint32_t *path_start;
    const uint8_t *fill_rule;
    const uint32_t *color;
    uint32_t n_points;
    uint32_t n_contours;
    uint32_t n_paths;
    float width;
    float height;
    uint32_t clear_color;
    const uint32_t *path_clip;   /* ABI 2 */
    const uint8_t *path_is_clip; /* ABI 2 */
    const pf_stroke *path_stroke;   /* ABI 3 */
    const uint8_t *contour_closed;  /* ABI 3 */
    const float *dashes;            /* ABI 3 */
    uint32_t n_dashes;              /* ABI 3 */
    const pf_paint *path_paint;     /* ABI 4 */
    const pf_color_stop *stops;     /* ABI 4 */
    uint32_t n_stops;               /* ABI 4 */
    const float *view_box;          /* ABI 5 */
    uint32_t load_action;           /* ABI 5 */
} pf_scene_view;

/* Context configuration.  Zero-initialise and set what you need. */
typedef struct pf_config {
    int device;            /* CUDA device ordinal                                */
    void *stream;          /* cudaStream_t to run on; NULL = context-owned stream */
    uint32_t flags;        /* PF_CONFIG_* bits                                    */
    uint32_t reserved[8];
} pf_config;

/* Per-frame counters (host copy).  Times are device milliseconds measured
 * with CUDA events when PF_CONFIG_STAGE_TIMING is set, else 0. */
typedef struct pf_frame_stats {
    uint64_t paths, contours, points, segments;
    uint64_t microlines;   /* flattened leaf lines (d3d9 recursion leaves)        */
    uint64_t tiles;        /* tiles in all path tile rects                         */
    uint64_t fills;        /* fills kept after culling                             */
    uint64_t alpha_tiles;  /* tiles holding at least one fill                      */
    uint64_t visible_tiles;/* alpha tiles plus solid tiles with a nonzero backdrop */
    uint64_t composite_entries; /* (framebuffer tile, path tile) pairs after z-cull */
    uint64_t framebuffer_tiles;
    uint32_t overflow;     /* nonzero if a predicted capacity overflowed and the   */
                           /* frame was re-run by the exact two-pass method        */
    uint32_t kernel_error; /* nonzero if a kernel hit an iteration bound            */
    float ms_setup, ms_flatten, ms_bin, ms_propagate, ms_lists, ms_composite, ms_total;
    uint64_t composited_fills; /* fills of the alpha tiles left in composite lists     */
    uint32_t kernel_launches;  /* CUDA kernels this frame launched                     */
    uint32_t host_syncs;       /* stream synchronisations this frame waited on        */
} pf_frame_stats;

#define PF_CONFIG_STAGE_TIMING 0x1u
/* Count the composite's work (entries, composited fills) and the draw paths' alpha and visible
 * tiles into pf_frame_stats; off by default because the counters cost a few atomics per block
 * and a pass over the tile states. */
#define PF_CONFIG_FRAME_COUNTERS 0x2u

/*
 * Canonical integer output of one scene (host memory, owned by the context
 * until the next call on it).  Tiles are numbered path-major and row-major
 * inside each path's tile rect (BuiltPath::tile_bounds,
 * pathfinder/core/data/built_path.cpp:8-34).  Fills are grouped by tile and
 * sorted inside a tile by (from_x, from_y, to_x, to_y) as u16.
 */
typedef struct pf_canon {
    uint32_t n_paths;
    const int32_t *path_rect;          /* [n_paths][4] x0,y0,x1,y1 tile rect    */
    const uint64_t *path_tile_first;   /* [n_paths + 1]                         */
    const uint64_t *path_column_first; /* [n_paths + 1]                         */
    uint64_t n_tiles;
    const uint8_t *tile_alpha;         /* [n_tiles] 1 = alpha tile              */
    const int8_t *tile_backdrop;       /* [n_tiles] propagated backdrop (int8)  */
    const uint32_t *tile_fill_count;   /* [n_tiles]                             */
    uint64_t n_fills;
    const uint16_t *fills;             /* [n_fills][4] from_x,from_y,to_x,to_y  */
    uint64_t n_columns;
    const int32_t *column_backdrop;    /* [n_columns] final column sums (int32) */
    uint32_t fb_tiles_x, fb_tiles_y;
    const int32_t *z;                  /* [fb tiles] topmost occluding path, -1 */
    const uint64_t *fb_list_first;     /* [fb tiles + 1]                        */
    uint64_t n_list;
    const uint32_t *fb_list;           /* global tile indices, back to front    */
    /* clipped draw tiles (ABI 2): 0 own mask, 1 the clip tile's mask (the draw tile was
     * solid), 2 own mask combined with the clip tile's; the clip tile (global index, or
     * UINT64_MAX) and, for 2, the draw tile's backdrop before it was zeroed */
    const uint8_t *tile_mask;          /* [n_tiles] */
    const uint64_t *tile_clip;         /* [n_tiles] */
    const int8_t *tile_dest_backdrop;  /* [n_tiles] */
} pf_canon;

/* Library and device queries. */
int pf_abi_version(void);
int pf_device_count(int *count);

/* Context lifetime. */
int pf_ctx_create(const pf_config *config, void **ctx);
int pf_ctx_destroy(void *ctx);
const char *pf_last_error(void *ctx);
int pf_ctx_set_flags(void *ctx, uint32_t flags); /* PF_CONFIG_* bits */

/*
 * Upload one scene (H2D copies on the context stream).  Replaces
 * SceneBuilderD3D11::build's CPU packing (pathfinder/core/d3d11/scene_builder.cpp:209-223):
 * segment extraction, bounds and tile rects are computed on the GPU.
 */
int pf_scene_upload(void *ctx, const pf_scene_view *scene);

/*
 * Upload a batch of independent scenes (each keeps its own canvas and image).
 * Host ranges that are contiguous across scenes are copied with one transfer.
 */
int pf_scene_upload_batch(void *ctx, const pf_scene_view *scenes, uint32_t n_scenes);

/*
 * Render the uploaded scene with the exact two-pass method (count, size,
 * write), leaving the RGBA8 image on the device.  Replaces
 * RendererD3D11::draw (pathfinder/core/d3d11/renderer.cpp:302-336).
 * stats may be NULL.
 */
int pf_render(void *ctx, pf_frame_stats *stats);

/* Same, for uploaded scenes [first_scene, first_scene + n_scenes) only: the
 * single-scene frame of the reference when n_scenes == 1. */
int pf_render_scenes(void *ctx, uint32_t first_scene, uint32_t n_scenes, pf_frame_stats *stats);

/*
 * The learned one-pass frame over uploaded scenes [first_scene, first_scene + n_scenes):
 * a per-path MLP (the "sizer", below) predicts every path's leaf-line and fill counts, the
 * frame lays out per-path leaf regions and the fill capacity from those predictions, and
 * flattens, stores and counts leaf lines in one pass (one host synchronisation after
 * set-up instead of the exact method's count-then-allocate passes).  Output is identical
 * to pf_render_scenes.  If a prediction is too small the frame is redone by the exact
 * method and stats->overflow is set.  Needs sizer weights (pf_sizer_load / _init).
 * The second such frame in a row over the same upload and scene range is recorded as a CUDA
 * graph and replayed, and later ones replay it (one launch, one synchronisation:
 * stats->host_syncs == 1) until the scenes, the sizer, the flags, the host image target or a
 * buffer changes.
 */
int pf_render_learned(void *ctx, uint32_t first_scene, uint32_t n_scenes, pf_frame_stats *stats);

/*
 * The frame to use by default: the learned frame where it pays, else the exact one.  The context
 * times both frames on the device over the workload (the scene range and its totals of paths,
 * contours and points: a later upload of scenes of the same size keeps what was measured) as they
 * run: the first calls run the exact frame until it has been timed twice, the next ones the
 * learned frame until it has been timed twice (neither frame's first run is timed, nor a learned
 * frame that records its CUDA graph; its replay is), and from then on the one whose faster timed
 * frame was faster: at most seven calls decide.  A learned frame that has to be redone exactly
 * (stats->overflow) counts as the slower one.  Without sizer weights every call runs the exact
 * frame.  Output is identical whichever runs.  No counterpart in the reference (its
 * count-then-allocate loop always runs, renderer.cpp:540-577).
 */
#define PF_FRAME_EXACT 0
#define PF_FRAME_LEARNED 1
int pf_render_auto(void *ctx, uint32_t first_scene, uint32_t n_scenes, pf_frame_stats *stats);
/* What pf_render_auto did: the frame its last call ran (PF_FRAME_*), the settled choice (-1 while
 * it is still timing), and each frame's fastest timed run (0 until timed). */
int pf_auto_choice(void *ctx, int *last, int *choice, float *exact_ms, float *learned_ms);

/*
 * Launch parameters of the frame's kernels (the configuration the autotuner searches; no
 * counterpart in the reference, whose dispatch sizes are fixed in its shaders).  Zero-initialise
 * and pf_tuning_get for the defaults.  Output never depends on them.
 */
typedef struct pf_tuning {
    uint32_t bin_ctas_per_sm[3]; /* binning CTAs resident per SM for the three CTA classes (paths
                                    whose rect plus a row of column sums takes <= 1088, 4352,
                                    16896 words); 0: as many as fit */
    float long_line;             /* lines spanning more tiles than this are walked by a whole warp */
    uint32_t bin_concurrent;     /* 1: the three binning classes run at once on side streams */
    uint32_t seg_sorted;         /* 1: the flatten takes segments ordered by subdivision depth */
    uint32_t composite_ticket;   /* 0: the composite runs a warp per framebuffer tile; n > 0: its warps
                                    stay resident and take n consecutive tiles per ticket from a
                                    frame-wide queue (at most 4096) */
    uint32_t reserved[8];
} pf_tuning;
int pf_tuning_get(void *ctx, pf_tuning *out);
int pf_tuning_set(void *ctx, const pf_tuning *tuning);
/*
 * Search the launch parameters on the uploaded scenes [first_scene, first_scene + n_scenes):
 * coordinate descent from the current parameters, each trial the default frame
 * (pf_render_auto's choice) run `frames` times and timed on the device (median), until no
 * parameter improves the frame by more than 1%.  The best parameters are left set; *best_ms and
 * *start_ms (the current parameters' time) may be NULL.  The caller persists them
 * (pathfinder-cpp_gb300/tune.py writes a RenderConfig JSON file).
 */
int pf_autotune(void *ctx, uint32_t first_scene, uint32_t n_scenes, uint32_t frames, pf_tuning *best, float *best_ms,
                float *start_ms);

/*
 * Learned sizer: features (12 per path) -> 64 -> 64 -> (log1p leaf lines, log1p fills),
 * bf16 weights, fp32 accumulation, trained on the GPU with the library's own forward,
 * backward and Adam kernels.  It replaces the reference's buffer sizing by readback and
 * retry (pathfinder/core/d3d11/renderer.cpp:540-577).  Budgets per path are
 * ceil(expm1(prediction) * mul + add); leaf lines past a path's budget spill into a shared
 * pool of pool_fraction x (sum of budgets) slots, and only an exhausted pool (or fills past
 * the summed fill estimate) sends the frame to the exact method.
 */
int pf_sizer_param_count(void);
int pf_sizer_init(void *ctx, uint64_t seed);
int pf_sizer_set_params(void *ctx, const float *params, size_t n);
int pf_sizer_get_params(void *ctx, float *params, size_t n);
int pf_sizer_set_margin(void *ctx, float mul, float add, float pool_fraction);
int pf_sizer_last_frame(void *ctx, uint32_t *paths_over_budget, uint32_t *pool_slots_used);
int pf_sizer_predict(void *ctx, const float *features, uint32_t n, float *out);

/*
 * Composite every later frame straight into host memory: `host` (at least pf_image_bytes bytes;
 * scene i's image at pf_image_offset(i)) receives the RGBA8 images over the GPU's coherent
 * link while the composite runs, so no copy follows the frame and pf_read_images into the same
 * buffer returns at once.  The buffer is pinned and mapped here (cudaHostRegister) unless the
 * caller pinned it already; NULL restores device-resident images.  No counterpart in the
 * reference (its destination is a GPU texture, Renderer::get_dest_texture,
 * pathfinder/core/renderer.h:82).
 */
int pf_set_host_image(void *ctx, void *host, size_t bytes);

/*
 * pf_sizer_predict without any device allocation, for callers that cannot call cudaMalloc
 * (a render loop that must not stall the device, or GPU memory owned by another allocator).
 * No counterpart in the reference.  It waits on the context's stream for its results before it
 * returns, as pf_sizer_predict does.  Features and
 * predictions are staged in a fixed device array of 16384 paths (about 0.9 MB, held by every
 * GPU that loads the library until exit); larger n is rejected with PF_ERR_INVALID_ARGUMENT.
 * Calls share the array: calls whose GPU work overlaps race; serialise them.
 * The context must already hold sizer weights.
 */
int pf_sizer_predict_noalloc(void *ctx, const float *features, uint32_t n, float *out);
int pf_sizer_gradient(void *ctx, const float *features, const float *targets, uint32_t n, float *grad,
                      float *loss);
int pf_sizer_train(void *ctx, const float *features, const float *targets, uint32_t n, uint32_t epochs,
                   uint32_t batch, float lr, uint64_t seed, float *epoch_losses);
int pf_sizer_save(void *ctx, const char *path);
int pf_sizer_load(void *ctx, const char *path);

/* Per-path features (n_paths x 12) and exact leaf-line / fill counts of the last frame
 * (the sizer's inputs and training labels). */
int pf_path_features(void *ctx, float *out, size_t capacity_floats);
int pf_path_counts(void *ctx, uint32_t *leaves, uint32_t *fills, size_t capacity);

/* The last frame's 16 status words: error bits, stage totals and counters (debug aid). */
int pf_debug_counters(void *ctx, uint32_t *out, size_t n);

/* Copy the last rendered image to host memory: RGBA8, row-major,
 * width_px * height_px * 4 bytes with width_px = ceil(width). */
int pf_read_image(void *ctx, uint8_t *rgba, size_t capacity_bytes);

/* Same for scene `scene` of an uploaded batch. */
int pf_read_image_scene(void *ctx, uint32_t scene, uint8_t *rgba, size_t capacity_bytes);

/* Every image of the uploaded batch in one copy: scene i's RGBA8 image starts at
 * byte offset_of(i) (pf_image_offset) of dst; the total is pf_image_bytes. */
int pf_image_bytes(void *ctx, uint64_t *bytes);
int pf_image_offset(void *ctx, uint32_t scene, uint64_t *offset);
int pf_read_images(void *ctx, uint8_t *dst, size_t capacity_bytes);

/*
 * The last frame's images to host memory without holding up the next frame: the images are
 * snapshotted on the device (on the context's stream) and copied to dst on a copy stream of the
 * context; the call returns at once, and later uploads and frames run while the copy does.
 * pf_images_wait blocks until the last such copy is complete; dst must not be read before.  A
 * later pf_read_images_async waits on the device for the previous copy before it snapshots
 * again.  With a host image target (pf_set_host_image) the images are already in host memory
 * and are copied to dst at once.  dst should be pinned for the copy to run asynchronously.
 */
int pf_read_images_async(void *ctx, uint8_t *dst, size_t capacity_bytes);
int pf_images_wait(void *ctx);

/*
 * Put pixels into scene `scene`'s destination image (RGBA8, width_px * height_px * 4 bytes, as
 * pf_read_image returns them), for a later frame with PF_LOAD_LOAD to composite over: the
 * reference's write into the destination texture (CommandEncoder::write_texture,
 * pathfinder/gpu/command_encoder.h) before Renderer::draw(..., clear_dst_texture = false).
 * Call it after the upload (an upload may reallocate the images).  Synchronises.
 */
int pf_write_image(void *ctx, uint32_t scene, const uint8_t *rgba, size_t bytes);

/* Device pointer and pitch of the last rendered image (valid until the next
 * render on this context). */
int pf_image_device_ptr(void *ctx, void **rgba, uint32_t *width_px, uint32_t *height_px);

/*
 * The fill outline of an uploaded scene, as the frames tile it: stroked paths replaced by
 * their stroke outlines (OutlineDash + OutlineStrokeToFill), other paths as uploaded.  Host
 * arrays owned by the context, valid until the next call on it (synchronises).
 */
typedef struct pf_outline {
    uint32_t n_points, n_contours, n_paths;
    const float *points;            /* [n_points][2] */
    const uint8_t *point_flags;     /* [n_points] */
    const uint32_t *contour_start;  /* [n_contours + 1] */
    const uint32_t *path_start;     /* [n_paths + 1] */
    const uint8_t *fill_rule;       /* [n_paths] (stroke outlines: PF_FILL_NONZERO) */
} pf_outline;
int pf_read_outline(void *ctx, uint32_t scene, pf_outline *out);

/* What the last upload's stroke pass did (all zero when it had no stroked path).  The device
 * times are taken when the context has PF_CONFIG_STAGE_TIMING. */
typedef struct pf_upload_stats {
    uint32_t n_points, n_contours;   /* the fill outline the frames tile (all scenes)   */
    uint32_t stroked_paths, dashed_paths;
    uint32_t stroke_contours;        /* output contours of the stroke pass (all paths)  */
    uint32_t dash_points;            /* points of the dashed contours                   */
    float ms_dash;                   /* device time of the dash kernels                 */
    float ms_stroke;                 /* device time of the stroke kernels               */
} pf_upload_stats;
int pf_upload_stats_get(void *ctx, pf_upload_stats *out);

/* Canonical integer output of the last rendered scene (synchronises). */
int pf_read_canon(void *ctx, pf_canon *out);
int pf_read_canon_scene(void *ctx, uint32_t scene, pf_canon *out);

/*
 * Coverage after the fill rule of every alpha tile of scene 0 of the last frame,
 * in tile order: *n_alpha x 256 floats (row-major 16x16).  With out == NULL only
 * *n_alpha is set.  A test and debugging aid (the frame itself never stores coverage).
 * A clipped tile is listed with its own mask, before the clip is applied.
 */
int pf_read_coverage(void *ctx, float *out, size_t capacity_floats, uint64_t *n_alpha);

/*
 * One call that uploads, renders and reads back: the per-frame work of
 * Canvas::draw (pathfinder/core/canvas.cpp:557-567) from host buffers to a
 * host image.
 */
int pf_draw(void *ctx, const pf_scene_view *scene, uint8_t *rgba, size_t capacity_bytes,
            pf_frame_stats *stats);

/*
 * SVG ingestion (host only, no device): the work of SvgScene::SvgScene
 * (pathfinder/core/svg.cpp:135-205): nanosvg's nsvgParse(text, "px", dpi) replayed through
 * the canvas.  Each shape gives a fill path (when its fill paint is visible) and a stroke path
 * (when its stroke paint is visible and its width positive), the stroke as the shape's
 * contours plus a pf_stroke the upload converts on the GPU (dashes at phase 0, as
 * Canvas::stroke_path dashes).  Colour, linear and radial gradient paints.  The text is copied;
 * the scene's arrays belong to the pf_svg and stay valid until pf_svg_free.  width and height
 * are the document's size in px.  A document without a shape gives a scene of no paths.
 */
typedef struct pf_svg pf_svg;
int pf_svg_parse(const char *text, size_t length, float dpi, pf_svg **out);
int pf_svg_scene(const pf_svg *svg, pf_scene_view *out);
void pf_svg_free(pf_svg *svg);

#ifdef __cplusplus
}
#endif

#endif /* PFCUDA_H */
