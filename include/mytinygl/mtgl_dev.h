/*
 * mtgl_dev.h — the thin C ABI between the C99 GL front end and a rendering back end.
 *
 * MyTinyGL rasterises synchronously inside glEnd (gl_api.c:635-662 → raster.c:901-1017).
 * Here glEnd, glDrawArrays and glDrawElements instead capture a *draw packet*: the
 * vertex source (client memory or a device buffer), the primitive mode and two state
 * blocks — the per-vertex state that emit_vertex reads (gl_api.c:263-348) and the raster
 * state that render_triangle / rasterize_triangle_smooth read (raster.c:451-958). The
 * packet crosses this ABI and the back end renders it in submission order.
 *
 * The CUDA back end (libmytinygl_gb300.so) queues packets and renders them with sm_103a
 * kernels when the frame is flushed. Every entry point returns an mtgl_status; the front
 * end turns failures into GL errors (GL_OUT_OF_MEMORY / GL_INVALID_OPERATION).
 * Only plain C types cross this boundary.
 */
#ifndef MYTINYGL_GB300_MTGL_DEV_H
#define MYTINYGL_GB300_MTGL_DEV_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define MTGL_MAX_LIGHTS 8

typedef enum {
    MTGL_OK = 0,
    MTGL_ERR_INVALID = 1,     /* bad argument or handle */
    MTGL_ERR_OOM = 2,         /* device or pinned-host allocation failed */
    MTGL_ERR_CUDA = 3,        /* a CUDA call failed; the message is in mtgl_dev_last_error() */
    MTGL_ERR_NO_DEVICE = 4,   /* no CUDA device is visible: the GPU back end never falls back */
    MTGL_ERR_UNSUPPORTED = 5, /* primitive or feature this back end does not render */
    MTGL_ERR_TIMEOUT = 6,     /* a bounded device-side wait gave up */
    MTGL_ERR_OVERFLOW = 7     /* a device work list exceeded its capacity (re-run with more) */
} mtgl_status;

typedef struct mtgl_dev mtgl_dev;  /* one per GL context: framebuffer + queue + resources */
typedef uint64_t mtgl_handle;      /* device buffer / texture handle; 0 means none */

/* One light, as stored by glLightfv (gl_api.c:1945-1995). position and spot_direction are
 * already in eye space. The last three derived fields are computed on the host with the
 * exact float operations compute_lighting performs per vertex (lighting.h:306-334), so the
 * device never re-derives them. */
typedef struct {
    float ambient[4], diffuse[4], specular[4];
    float position[4];
    float spot_direction[3];
    float spot_exponent, spot_cutoff;
    float constant_attenuation, linear_attenuation, quadratic_attenuation;
    float dir_normalized[3];       /* vec3_normalize(position.xyz), directional lights   */
    float spot_dir_normalized[3];  /* vec3_normalize(spot_direction)                     */
    float cos_cutoff;              /* cosf(spot_cutoff * 3.14159265f / 180.0f)          */
    uint32_t enabled;
} mtgl_light;

/* material_t (mytinygl.h:69-75) */
typedef struct {
    float ambient[4], diffuse[4], specular[4], emission[4];
    float shininess;
} mtgl_material;

/* Everything compute_lighting reads (lighting.h:284-373). */
typedef struct {
    mtgl_light lights[MTGL_MAX_LIGHTS];
    mtgl_material front, back;
    float model_ambient[4];
    uint32_t local_viewer, two_side, normalize;
} mtgl_lighting;

/* Per-vertex state: what emit_vertex reads at the moment of each glVertex call. */
typedef struct {
    float modelview[16], projection[16], texture[16];
    float normal_matrix[16];       /* mat4_normal_matrix(modelview), graphics.h:229-260 */
    uint32_t lighting;             /* GL_LIGHTING enabled                               */
    uint32_t color_material;       /* GL_COLOR_MATERIAL enabled                         */
    uint32_t color_material_face, color_material_mode;
    uint32_t phong;                /* shade model GL_PHONG: no per-vertex lighting       */
    uint32_t pad_;
    mtgl_lighting lit;
} mtgl_vertex_state;

/* Raster state: what render_triangle and rasterize_triangle_smooth read at glEnd. */
typedef struct {
    int32_t viewport[4];           /* x, y, w, h (framebuffer y grows downwards)          */
    int32_t scissor[4];
    uint32_t scissor_test;
    uint32_t depth_test, depth_func, depth_mask;
    double depth_near, depth_far;
    uint32_t stencil_test, stencil_func;
    int32_t stencil_ref;
    uint32_t stencil_mask, stencil_fail, stencil_zfail, stencil_zpass, stencil_writemask;
    uint32_t blend, blend_src, blend_dst;
    uint32_t alpha_test, alpha_func;
    float alpha_ref;
    uint32_t color_mask[4];
    uint32_t cull_face, cull_face_mode, front_face;
    uint32_t polygon_mode_front, polygon_mode_back;
    uint32_t shade_model, perspective_hint;
    uint32_t fog, fog_mode;
    float fog_density, fog_start, fog_end, fog_color[4];
    uint32_t tex_env_mode;
    float tex_env_color[4];
    mtgl_handle texture;           /* 0: no texturing (disabled, unbound or no image)    */
    int32_t tex_min_filter, tex_mag_filter, tex_wrap_s, tex_wrap_t;
    float line_width, point_size;
    uint32_t lighting;             /* GL_LIGHTING at glEnd (per-fragment paths)           */
    uint32_t pad_;
    mtgl_lighting lit;             /* lights/materials at glEnd (GL_PHONG, two-sided)     */
} mtgl_raster_state;

/* One vertex attribute stream, resolved by the front end at draw time
 * (get_array_pointer / get_array_element, gl_api.c:1745-1797). */
typedef struct {
    const void *host;              /* client memory, borrowed for the call only           */
    mtgl_handle buffer;            /* or a device buffer ...                              */
    uint64_t offset;               /* ... at this byte offset                             */
    uint64_t bytes;                /* readable bytes from the start (bounds for fetches)  */
    int32_t size, type, stride;    /* components, GL_FLOAT/GL_UNSIGNED_BYTE, byte stride  */
    int32_t enabled;               /* 0: the attribute comes from the current value       */
} mtgl_attrib;

/* One draw: a glBegin/glEnd batch or one glDrawArrays / glDrawElements call. */
typedef struct {
    uint32_t mode;                 /* GL_POINTS .. GL_POLYGON                             */
    int32_t first;                 /* glDrawArrays: first element index                   */
    int32_t count;                 /* number of elements                                  */
    uint32_t index_type;           /* 0, GL_UNSIGNED_BYTE, _SHORT or _INT                 */
    const void *index_host;        /* client indices (borrowed for the call), or ...      */
    mtgl_handle index_buffer;      /* ... a device element buffer                         */
    uint64_t index_offset;
    int64_t index_min, index_max;  /* non-negative index range (front end computes)       */
    int32_t has_negative_index;    /* an index >= 2^31 reads the default attributes       */
    int32_t position_2d;           /* glVertex2f: z = 0 (vertex array size 2)             */
    mtgl_attrib position, color, texcoord, normal;
    float current_color[4], current_texcoord[2], current_normal[3];
    /* Immediate mode: vertex i uses vertex_states[vertex_state_ids[i]]. When
     * vertex_state_ids is NULL every vertex uses vertex_states[0]. */
    const uint32_t *vertex_state_ids;
    const mtgl_vertex_state *vertex_states;
    uint32_t vertex_state_count;
    const mtgl_raster_state *raster_state;
} mtgl_draw;

/* Counters since the last mtgl_dev_reset_stats. */
typedef struct {
    uint64_t draws, input_triangles, setup_triangles, bin_entries, fragments;
    uint64_t passes, kernel_launches;
    uint64_t staged_bytes;         /* client data (attributes, indices, state ids) staged */
    uint64_t allocations;          /* device or page-locked allocations made for this context's
                                      passes (scratch, staging areas) */
    uint64_t vertices;             /* vertex slots transformed by the vertex stage */
    uint64_t vertex_bytes;         /* attribute bytes those slots read (enabled arrays) */
    uint64_t debug_status;         /* build with MTGL_DEBUG_BOUNDS: the site code of the first
                                      device index check that failed (0: none). Any build: 7
                                      when a scan's bounded wait for an earlier block ran out
                                      (never expected; the pass's results are then wrong) */
} mtgl_stats;

/* Device time per pipeline phase, summed over the passes since profiling was enabled
 * (CUDA events recorded on the context's stream around each phase). */
typedef struct {
    double vertex_ms, setup_ms, bin_ms, tile_ms;
    uint64_t passes;
} mtgl_timings;

/* ---- lifetime ---- */
int mtgl_dev_create(int32_t width, int32_t height, mtgl_dev **out);
int mtgl_dev_destroy(mtgl_dev *d);
const char *mtgl_dev_last_error(void);
const char *mtgl_dev_backend_name(void);

/* ---- resources (replace textures.c / vbo.c storage) ---- */
int mtgl_dev_buffer_create(mtgl_dev *d, mtgl_handle *out);
int mtgl_dev_buffer_data(mtgl_dev *d, mtgl_handle h, const void *data, uint64_t bytes);
int mtgl_dev_buffer_sub_data(mtgl_dev *d, mtgl_handle h, uint64_t offset, const void *data, uint64_t bytes);
int mtgl_dev_buffer_destroy(mtgl_dev *d, mtgl_handle h);
int mtgl_dev_texture_create(mtgl_dev *d, mtgl_handle *out);
/* rgba32: packed a<<24|b<<16|g<<8|r texels (graphics.h:420-434). Builds mip level 1. */
int mtgl_dev_texture_image(mtgl_dev *d, mtgl_handle h, int32_t width, int32_t height, const uint32_t *rgba32);
int mtgl_dev_texture_destroy(mtgl_dev *d, mtgl_handle h);
/* Replace level `level` (>= 1) of a texture whose chain was built under
 * MTGL_OPT_MIPMAP_CHAIN; the size must be the level's. No counterpart in the reference.
 * Returns MTGL_ERR_INVALID when the texture has no such level or the size differs. */
int mtgl_dev_texture_level(mtgl_dev *d, mtgl_handle h, int32_t level, int32_t width, int32_t height,
                           const uint32_t *rgba32);

/* ---- commands, executed in submission order ---- */
/* glClear over [x0,x1) x [y0,y1) (already clamped), gl_api.c:409-457 */
int mtgl_dev_clear(mtgl_dev *d, uint32_t mask, int32_t x0, int32_t y0, int32_t x1, int32_t y1,
                   uint32_t color, float depth, uint8_t stencil);
int mtgl_dev_draw(mtgl_dev *d, const mtgl_draw *draw);
/* glDrawPixels (gl_api.c:1287-1376): rgba32 is width*height packed texels, bottom row first. */
int mtgl_dev_draw_pixels(mtgl_dev *d, int32_t raster_x, int32_t raster_y, int32_t width, int32_t height,
                         const uint32_t *rgba32, const mtgl_raster_state *rs);

/* ---- synchronisation and readback ---- */
int mtgl_dev_flush(mtgl_dev *d);   /* submit queued work; returns without waiting        */
int mtgl_dev_finish(mtgl_dev *d);  /* submit and wait                                    */
/* 1 while a batch that writes this context's framebuffer or reads its resources has not
 * been waited for (by mtgl_dev_batch_wait, or by an operation of the context that needs
 * it), else 0. A context at 0 shares no host state with other contexts until it joins a
 * batch, so distinct such contexts can be driven from distinct threads (mtgl_play_many). */
int mtgl_dev_in_batch(const mtgl_dev *d);
/* Finish, then copy whole buffers (row 0 = top) to host memory; any pointer may be NULL. */
int mtgl_dev_read(mtgl_dev *d, uint32_t *color, float *depth, uint8_t *stencil);
int mtgl_dev_stats(mtgl_dev *d, mtgl_stats *out);
/* 1 in a build with MTGL_DEBUG_BOUNDS (device index checks that record a failing site in
 * mtgl_stats.debug_status and skip the access, never trapping), else 0. No counterpart in
 * the reference, whose framebuffer accessors can only have their checks removed
 * (framebuffer.h:92-163). */
int mtgl_dev_debug_bounds(void);
int mtgl_dev_reset_stats(mtgl_dev *d);
/* Per-phase device timing (off by default); enabling resets the sums. */
int mtgl_dev_profile(mtgl_dev *d, int enable);
int mtgl_dev_timings(mtgl_dev *d, mtgl_timings *out);
/* The cudaStream_t every operation of this context runs on (NULL for a CPU back end). */
void *mtgl_dev_stream(mtgl_dev *d);

/* Per-context options. MTGL_OPT_DEPTH_REJECTION (default 1): the tile kernel skips, per
 * warp, triangles none of whose fragments can pass GL_LESS/GL_LEQUAL/GL_NEVER while the
 * stencil test is off. Rendering is identical either way; with it off every covered
 * fragment is counted in mtgl_stats.fragments. Applies to draws queued afterwards. */
#define MTGL_OPT_DEPTH_REJECTION 1
/* MTGL_OPT_MIPMAP_CHAIN (default 0): an extension with no counterpart in MyTinyGL, whose
 * glTexImage2D accepts level 0 only and whose sampler knows level 0 and one derived level
 * (textures.c:311-354, 457-557). With it on, a texture image given afterwards also gets
 * every further level (each a 2x2 box filter of the one before, down to a side of 1),
 * glTexImage2D accepts levels above 0 of matching size (replacing that level), and the
 * mipmap filters use the whole chain: GL_*_MIPMAP_NEAREST the level nearest the triangle's
 * LOD, GL_*_MIPMAP_LINEAR a blend of the two levels around it. Rendering is then outside
 * parity with the reference (which clamps the LOD to level 1); with it off nothing changes. */
#define MTGL_OPT_MIPMAP_CHAIN 2
int mtgl_dev_set_option(mtgl_dev *d, int option, int value);

/* ---- batches: many contexts' pending passes in one pipeline run ----
 *
 * No counterpart in MyTinyGL, which renders one context at a time inside glEnd. A batch
 * takes the pending pass (clears, then draws) of each of n contexts of one device, each
 * with its own framebuffer size and GL state, and renders them all with one run of the
 * pipeline: one vertex launch, one setup launch, one binning pass over the tiles of all
 * frames, and one persistent tile launch whose CTAs take (frame, tile) work items from a
 * device queue, costliest first. The run enqueues without host waits and is captured in a
 * CUDA graph, replayed while the batch keeps its shape. Every framebuffer ends up exactly
 * as rendering each context alone would leave it.
 *
 * Record and tile-pair buffers have fixed capacities (set from the config, then from the
 * largest totals seen). A run that exceeds one leaves every framebuffer untouched;
 * mtgl_dev_batch_wait sees it, grows the capacities and renders the batch again. */
typedef struct mtgl_batch mtgl_batch;

typedef struct {
    int32_t tile_size;       /* 8, 16 or 32 pixels; 0: the tuned default                    */
    int32_t ctas_per_sm;     /* persistent tile CTAs per SM; 0: the tuned default           */
    float record_factor;     /* initial record capacity per input triangle; 0: default      */
    float pair_factor;       /* initial tile-pair capacity per record; 0: default           */
    int32_t use_graph;       /* 1: capture the run in a CUDA graph and replay it; 0: launch */
    int32_t order_by_cost;   /* 1: hand out the costliest tiles first; 0: in frame order    */
    int32_t readback_kernel; /* 1: colour read-backs into mapped page-locked host memory are
                                written by a kernel (one launch per 128 frames); 0: one copy
                                call per frame. Other destinations are always copied.       */
} mtgl_batch_config;

typedef struct {
    uint64_t batches, frames, input_triangles, setup_triangles, bin_entries, fragments;
    uint64_t graph_captures, graph_replays, overflow_reruns, kernel_launches;
    uint32_t record_capacity, pair_capacity;
    int32_t tile_size, ctas;
    uint64_t vertices, vertex_bytes; /* as in mtgl_stats, over the batch's passes */
    uint64_t debug_status;           /* as in mtgl_stats */
} mtgl_batch_stats;

/* The defaults mtgl_dev_batch_create uses for zero fields. */
void mtgl_dev_batch_defaults(mtgl_batch_config *cfg);
int mtgl_dev_batch_create(const mtgl_batch_config *cfg, mtgl_batch **out);
int mtgl_dev_batch_destroy(mtgl_batch *b);
/* Renders the pending pass of each of devs[0..n) (each context at most once) as one
 * batch and returns without waiting; a previous submission of b is waited for first.
 * Afterwards each context reads, flushes or changes resources only after the batch. */
int mtgl_dev_batch_submit(mtgl_batch *b, mtgl_dev *const *devs, int32_t n);
/* The same, step by step: begin (waits for the previous submission), then any number of
 * add (src's pending pass, recorded on src with its resources, renders into target's
 * framebuffer; targets are distinct within a batch, a source may give several passes),
 * readback (after the run, copy target's colour buffer to host memory; page-locked memory
 * keeps the copy asynchronous), then launch. */
int mtgl_dev_batch_begin(mtgl_batch *b);
int mtgl_dev_batch_add(mtgl_batch *b, mtgl_dev *src, mtgl_dev *target);
int mtgl_dev_batch_readback(mtgl_batch *b, mtgl_dev *target, uint32_t *host_color);
int mtgl_dev_batch_launch(mtgl_batch *b);
/* Waits for the last submission and checks its capacities (see above). */
int mtgl_dev_batch_wait(mtgl_batch *b);
/* 1 when the last submission has finished on the device (mtgl_dev_batch_wait then returns
 * without blocking unless the run overflowed), 0 while it runs, negative on error. */
int mtgl_dev_batch_query(mtgl_batch *b);
int mtgl_dev_batch_stats(mtgl_batch *b, mtgl_batch_stats *out);
int mtgl_dev_batch_reset_stats(mtgl_batch *b);
/* The cudaStream_t the batch runs on. */
void *mtgl_dev_batch_stream(mtgl_batch *b);
/* Per-phase device timing of the batch's runs, as mtgl_dev_profile / mtgl_dev_timings.
 * Runs replayed from a CUDA graph carry no phase events: profile with use_graph = 0. */
int mtgl_dev_batch_profile(mtgl_batch *b, int enable);
int mtgl_dev_batch_timings(mtgl_batch *b, mtgl_timings *out);

#ifdef __cplusplus
}
#endif

#endif /* MYTINYGL_GB300_MTGL_DEV_H */
