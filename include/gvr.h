/*
 * gvr.h — C ABI of the GB300 volume renderer (Ascent scene plot `type: volume`).
 *
 * Every entry point is `extern "C"`, takes plain pointers and sizes, and
 * returns a gvr_status. The message of the last failing call on the calling
 * host thread is available from gvr_last_error().
 *
 * Conventions shared by every call:
 *   - Images are row-major, pixel_id = y * width + x, y pointing up (the
 *     VTK-m canvas convention that VolumeRenderer.cpp:299-300 decodes).
 *   - Colours are RGBA float32, premultiplied by alpha.
 *   - Depth is the image-space depth 0.5 * z_ndc + 0.49 of the front-most
 *     volume partial (src/libs/vtkh/rendering/VolumeRenderer.cpp:369-372);
 *     pixels that no partial reaches keep gvr_render_params.clear_depth.
 *   - `stream` is a cudaStream_t passed as void*; NULL means the legacy
 *     default stream. Calls are stream-ordered; host outputs are complete
 *     when the call returns.
 *   - GVR_MEM_HOST / GVR_MEM_DEVICE say where a caller buffer lives.
 *   - A gvr_scene is used by one host thread at a time. Different scenes
 *     may be driven from different threads at once: each has its own
 *     device state, staging buffers, copy stream and timeout flag, and the
 *     library's shared scratch pool and launch counter are thread-safe.
 */
#ifndef GVR_H
#define GVR_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define GVR_VERSION 1

#if defined(GVR_BUILDING) && defined(__GNUC__)
#define GVR_API __attribute__((visibility("default")))
#else
#define GVR_API
#endif

typedef enum gvr_status {
  GVR_OK = 0,
  GVR_ERR_INVALID_ARGUMENT = 1,
  GVR_ERR_CUDA = 2,
  GVR_ERR_OUT_OF_MEMORY = 3,
  GVR_ERR_UNSUPPORTED = 4,
  GVR_ERR_TIMEOUT = 5,      /* a bounded device-side wait gave up */
  GVR_ERR_NOT_FOUND = 6
} gvr_status;

enum { GVR_MEM_HOST = 0, GVR_MEM_DEVICE = 1 };
enum { GVR_DTYPE_FLOAT32 = 0, GVR_DTYPE_FLOAT64 = 1 };
enum { GVR_ASSOC_VERTEX = 0, GVR_ASSOC_ELEMENT = 1 };
enum { GVR_DOMAIN_UNIFORM = 0, GVR_DOMAIN_RECTILINEAR = 1, GVR_DOMAIN_HEX = 2 };
enum { GVR_LUT_NEAREST = 0, GVR_LUT_LINEAR = 1 };
enum { GVR_UINT8_NONE = 0, GVR_UINT8_ROUND = 1, GVR_UINT8_TRUNCATE = 2 };

/* A perspective camera (the state vtkm::rendering::Camera keeps in 3D mode,
 * as set by parse_camera, ascent_runtime_conduit_to_vtkm_parsing.cpp:91-174).
 * fov_y is in degrees; zoom is the multiplicative factor Ascent's `zoom` key
 * gives after zoom_to_vtkm_zoom (conduit_to_vtkm_parsing.cpp:59-69), i.e.
 * 1 means no zoom; xpan/ypan shift the image in normalised device units. */
typedef struct gvr_camera {
  float position[3];
  float look_at[3];
  float up[3];
  float fov_y;
  float zoom;
  float xpan;
  float ypan;
  float near_plane;
  float far_plane;
} gvr_camera;

/* Parameters of one volume render (VolumeRenderer::PreExecute and the
 * per-domain wrappers, VolumeRenderer.cpp:93-284, 600-612). */
typedef struct gvr_render_params {
  int width;
  int height;
  float sample_dist;        /* world units between samples along a ray     */
  float scalar_min;         /* m_range after Renderer::PreExecute          */
  float scalar_max;
  const float *lut_rgba;    /* host pointer, lut_size RGBA entries          */
  int lut_size;             /* 1 .. 4096                                    */
  int lut_filter;           /* GVR_LUT_NEAREST or GVR_LUT_LINEAR            */
  float alpha_cull;         /* partials with alpha below this are dropped
                               (0.001f, VolumeRenderer.cpp:271)             */
  float early_term;         /* stop a ray once its alpha reaches this;
                               >= 1 disables early termination              */
  int quantize_uint8;       /* 1: round-trip the canvas through the uint8
                               vtkh::Image (Image.hpp:102-105)              */
  int render_bg;            /* blend bg_color behind the volume             */
  float bg_color[4];
  float clear_depth;        /* depth of pixels no partial reaches           */
} gvr_render_params;

/* A 1D colour/opacity transfer function given as control points
 * (parse_color_table, conduit_to_vtkm_parsing.cpp:199-305). Positions are
 * normalised scalars in [0,1], sorted ascending and unique. */
typedef struct gvr_color_table {
  int n_rgb;
  const double *rgb_pos;    /* n_rgb positions                              */
  const double *rgb;        /* 3 * n_rgb colours in [0,1]                   */
  int n_alpha;
  const double *alpha_pos;  /* n_alpha positions                            */
  const double *alpha;      /* n_alpha opacities in [0,1]                   */
} gvr_color_table;

typedef struct gvr_scene gvr_scene;

/* ------------------------------------------------------------------ */
/* Library                                                              */
/* ------------------------------------------------------------------ */

/* Message of the last failing call on this host thread ("" if none). */
GVR_API const char *gvr_last_error(void);

/* GVR_VERSION of the loaded library. */
GVR_API int gvr_version(void);

/* Number of CUDA kernels this library has launched since it was loaded
 * (a diagnostic; no counterpart in the reference). */
GVR_API int gvr_launch_count(uint64_t *n);

/* ------------------------------------------------------------------ */
/* Host logic of the volume plot (no device work)                       */
/* ------------------------------------------------------------------ */

/* Opacity correction of every alpha control point:
 * a' = 1 - (1 - a)^(10 / num_samples).
 * Replaces VolumeRenderer::CorrectOpacity (VolumeRenderer.cpp:448-466).
 * Errors: num_samples < 1 (VolumeRenderer::SetNumberOfSamples, :622-629). */
GVR_API int gvr_correct_opacity(const double *alpha_in, int n, int num_samples,
                        double *alpha_out);

/* sample_dist = |extent(bounds)| / num_samples, bounds = {xmin,xmax,ymin,
 * ymax,zmin,zmax}. Replaces VolumeRenderer::PreExecute (:600-612). */
GVR_API int gvr_sample_distance(const double bounds[6], int num_samples,
                        float *sample_dist);

/* Sample the transfer function at n evenly spaced positions i/(n-1) into
 * n RGBA floats. uint8_mode GVR_UINT8_ROUND/TRUNCATE passes every channel
 * through an 8-bit value and back (x/255), as detail::convert_table does for
 * the multi-domain path (VolumeRenderer.cpp:65-90, 1024 entries). */
GVR_API int gvr_color_table_sample(const gvr_color_table *table, int n,
                           int uint8_mode, float *rgba_out);

/* Default camera for the scene bounds (vtkm Camera::ResetToBounds, called
 * by vtkh::MakeRender, Render.cpp:314-347). */
GVR_API int gvr_camera_reset_to_bounds(gvr_camera *camera, const double bounds[6]);

/* Rotate the camera position about the view-up axis through look_at
 * (parse_camera `azimuth`, conduit_to_vtkm_parsing.cpp:165-169). */
GVR_API int gvr_camera_azimuth(gvr_camera *camera, double degrees);

/* Rotate the camera position about the right axis through look_at
 * (parse_camera `elevation`, conduit_to_vtkm_parsing.cpp:170-174). */
GVR_API int gvr_camera_elevation(gvr_camera *camera, double degrees);

/* Cinema sweep cameras: one camera per (phi, theta) pair in degrees,
 * phi_theta holding 2*n floats. Replaces
 * CinemaManager::create_cinema_cameras
 * (ascent_runtime_rendering_filters.cpp:906-960). */
GVR_API int gvr_cinema_cameras(const double bounds[6], const float *phi_theta, int n,
                       gvr_camera *cameras_out);

/* Visibility order of n domains for one camera: order[d] is the rank of
 * domain d when domains are sorted by the distance from the camera to the
 * centre of their bounds (6 doubles per domain). Replaces
 * VolumeRenderer::FindVisibilityOrdering / FindMinDepth / DepthSort
 * (VolumeRenderer.cpp:638-650, 691-831, 834-866). */
GVR_API int gvr_visibility_order(const gvr_camera *camera, const double *domain_bounds,
                         int n, int *order);

/* ------------------------------------------------------------------ */
/* Device-resident scene                                                */
/* ------------------------------------------------------------------ */

/* Create an empty scene whose domains live on CUDA device `device`.
 * Replaces the vtkh::DataSet handed to VolumeRenderer::SetInput
 * (VolumeRenderer.cpp:868-907). */
GVR_API int gvr_scene_create(int device, gvr_scene **scene_out);
GVR_API int gvr_scene_destroy(gvr_scene *scene);

/* Add a uniform domain: dims = node counts (>= 2 each), origin/spacing
 * cast to float32 as the Blueprint adapter does
 * (ascent_vtkh_data_adapter.cpp:1177-1313). The scalar field has
 * dims[0]*dims[1]*dims[2] values (vertex) or (dims-1) products (element),
 * x fastest, `stride` elements apart (1 = contiguous), in `location`
 * memory, float32 or float64 (AddField, :1782-2040). The field is copied
 * into the scene's bricked device layout. */
GVR_API int gvr_scene_add_uniform(gvr_scene *scene, const int dims[3],
                          const double origin[3], const double spacing[3],
                          const void *field, int dtype, int64_t stride,
                          int association, int location, int *domain_id);

/* Add a rectilinear domain with per-axis node coordinates x[dims[0]],
 * y[dims[1]], z[dims[2]] (host, strictly increasing;
 * RectilinearBlueprintToVTKmDataSet, ascent_vtkh_data_adapter.cpp:1318-1430). */
GVR_API int gvr_scene_add_rectilinear(gvr_scene *scene, const int dims[3],
                              const double *x, const double *y, const double *z,
                              const void *field, int dtype, int64_t stride,
                              int association, int location, int *domain_id);

/* Add an unstructured hexahedral domain: n_nodes node coordinates in three
 * arrays x, y, z (float32 or float64, Blueprint explicit coordset), n_cells
 * cells of 8 node ids each in VTK hexahedron order (int32, or int64 when
 * conn_int64), and a scalar field per node (vertex) or per cell (element).
 * All arrays are in `location` memory. The domain's LBVH (Morton codes,
 * Karras radix tree, box refit), face-neighbour table and per-cell
 * monomial coefficients of the trilinear map (which the march evaluates)
 * are built on the device. Replaces the
 * unstructured path of the Blueprint adapter
 * (ascent_vtkh_data_adapter.cpp:1618-1780) and the ConnectivityProxy set-up
 * of VolumeRenderer's UnstructuredWrapper (VolumeRenderer.cpp:182-220). */
GVR_API int gvr_scene_add_hex(gvr_scene *scene, int64_t n_nodes, const void *x,
                              const void *y, const void *z, int coord_dtype,
                              int64_t n_cells, const void *conn, int conn_int64,
                              const void *field, int dtype, int association,
                              int location, int *domain_id);

/* Copy a hex domain's LBVH to host arrays (any may be NULL): sorted Morton
 * codes and leaf cell ids (n_cells each), Karras children left/right
 * (n_cells-1; values >= n_cells-1 are leaves n - (n_cells-1)), parents
 * (2 n_cells - 1, root -1), inner boxes (6 floats lo xyz, hi xyz per inner
 * node) and the build's wall time in ms. For checking the build against a
 * CPU rebuild (Devil Ray's LinearBVHBuilder, linear_bvh_builder.cpp:60-520). */
GVR_API int gvr_scene_hex_bvh(const gvr_scene *scene, int domain_id, uint32_t *codes,
                              uint32_t *ids, int32_t *left, int32_t *right,
                              int32_t *parent, float *inner_boxes, float *build_ms);

/* Copy a hex domain's face-neighbour table to the host: 6 cell ids per cell
 * (faces r=0, r=1, s=0, s=1, t=0, t=1 of the VTK hexahedron; -1 where the
 * face is on the boundary), built on the device at ingest from a sort of the
 * faces by their node ids. The march steps along it from cell to cell
 * before falling back to the LBVH, as VTK-m's unstructured tracer walks
 * cell faces (ConnectivityProxy, VolumeRenderer.cpp:182-220). build_ms (may
 * be NULL) receives the build's wall time. */
GVR_API int gvr_scene_hex_neighbors(const gvr_scene *scene, int domain_id, int32_t *nbr,
                                    float *build_ms);

/* Locate n points (3 n host floats) in a hex domain: cells[i] = containing
 * cell or -1, rst = reference coordinates (Devil Ray's DeviceMesh::locate,
 * data_model/device_mesh.hpp:250-360, with NewtonSolve). */
GVR_API int gvr_scene_hex_locate(gvr_scene *scene, int domain_id, const float *points,
                                 int n, int *cells, float *rst);

/* Replace the field of an existing domain (same size, type rules as the
 * add call); the bricked copy and macrocell ranges (hexahedral domains: the
 * node values and cell coefficients) are rebuilt on the device. */
GVR_API int gvr_scene_update_field(gvr_scene *scene, int domain_id, const void *field,
                           int dtype, int64_t stride, int location);

/* Replace the fields of n domains in one call (each as
 * gvr_scene_update_field would, same dtype/stride/location for all) — the
 * per-domain AddField loop of the Blueprint adapter when a simulation
 * publishes a new time step (ascent_vtkh_data_adapter.cpp:1782-2040). Host
 * fields are copied on a copy stream into staging buffers (up to one per
 * domain, 8 at most, about 1 GB in all) while earlier domains are bricked
 * on `stream`; ranges are reduced on the device and read back once. Host
 * fields in pinned memory overlap best. Returns after the uploads are
 * complete.
 *
 * Contiguous float32 fields are bricked from shared memory filled by bulk
 * async copies, which the kernel waits for with a bounded wait. If that wait
 * gives up, the bricks are written with non-finite ranges, the call (and
 * gvr_scene_update_field / the add calls) returns GVR_ERR_TIMEOUT, and the
 * domains' ranges stay NaN until the fields are published again. The
 * environment variable GVR_STAGE_WAIT_POLLS (0 .. 4194304, default the
 * maximum) sets the first wait's poll limit; 0 exercises that path. */
GVR_API int gvr_scene_update_fields(gvr_scene *scene, int n, const int *domain_ids,
                                    const void *const *fields, int dtype, int64_t stride,
                                    int location, void *stream);

GVR_API int gvr_scene_num_domains(const gvr_scene *scene, int *n);

/* Launch shape of the scene's march kernel: pixel packet width per warp
 * (4, 8 or 16; the packet is 32 rays), samples located per loop iteration
 * (1 to 4; 16-wide packets at most 3, and 3 only with min_blocks 4; the
 * batch path uses 2 for more) and CTAs per SM targeted by the register
 * budget (3 or 4). Results do not depend on it.
 * Set by the autotuner (ascent_gb300.tune); no counterpart in the
 * reference. */
GVR_API int gvr_scene_set_tuning(gvr_scene *scene, int packet_w, int unroll,
                                 int min_blocks);

/* Brick size of the vertex fields this scene bricks from now on: 4, 8
 * (default) or 16 cells per axis, so bricks of 5^3, 9^3 or 17^3 nodes
 * (1.95x, 1.42x or 1.20x the field) and an empty-space map of that
 * granularity. Call it before adding vertex-field domains (an error
 * otherwise). Images do not depend on it. Set by the autotuner
 * (ascent_gb300.tune.autotune_bricks); the reference keeps VTK-m's
 * unbricked arrays, so no counterpart. */
GVR_API int gvr_scene_set_brick_cells(gvr_scene *scene, int cells);

/* How the plain march reads bricks: mode 0 gathers each sample's corners
 * through the L1 cache; mode 1 stages, per 16 x 16 tile and slab of ray
 * distance, the bricks the tile's rays cross into shared memory with bulk
 * async copies and reads them there; mode 2 walks each domain's brick
 * layers along the rays' dominant axis, bulk-copying each layer's window of
 * bricks into one of two shared-memory buffers while the rays sample the
 * other (modes 1 and 2: scenes of uniform vertex-field domains in 8^3-cell
 * bricks only; other scenes, and the batch path, use mode 0; mode 2 also
 * leaves scenes with empty bricks to jump to the gather). Images are the
 * same in every mode. Set by the autotuner (ascent_gb300.tune); the march the
 * reference runs is VTK-m's (VolumeRenderer.cpp:258, 523-528), so no
 * counterpart. */
GVR_API int gvr_scene_set_staging(gvr_scene *scene, int mode);

/* Launch order of the plain march's 16 x 16 tiles: mode 0 (default) takes
 * the tiles nearest the image centre first, from a table built once per
 * image size; mode 1 runs, before every render, two small kernels that
 * estimate each tile's cost for that view (the length of five of its rays
 * inside the domain boxes) and sort the tiles, longest first. Images are
 * the same either way. Renders of one scene share the mode-1 order buffer,
 * like its transfer-function state: do not overlap them on different
 * streams. Set by the autotuner; no counterpart in the reference. */
GVR_API int gvr_scene_set_tile_order(gvr_scene *scene, int mode);

/* Number of tiles whose bounded wait for their staged bricks gave up since
 * the scene was created (each finished from global memory; 0 normally). */
GVR_API int gvr_scene_staging_failures(const gvr_scene *scene, uint64_t *n);

/* Bounds {xmin,xmax,ymin,ymax,zmin,zmax} of one domain, or of the whole
 * scene when domain_id == -1 (DataSet::GetGlobalBounds). */
GVR_API int gvr_scene_bounds(const gvr_scene *scene, int domain_id, double bounds[6]);

/* Global scalar range {min,max} of the scene field (Renderer::PreExecute,
 * Renderer.cpp:144-179). Both NaN while a domain's last field publish
 * returned GVR_ERR_TIMEOUT (publish the field again). */
GVR_API int gvr_scene_range(const gvr_scene *scene, double range[2]);

/* ------------------------------------------------------------------ */
/* Rendering                                                            */
/* ------------------------------------------------------------------ */

/* Render the scene's volume for one camera into rgba (4*W*H floats) and
 * depth (W*H floats), both in `out_location` memory. Each ray visits the
 * domains it crosses in increasing entry distance (each from the furthest
 * exit reached so far) and composites their partials front to back, as the
 * reference's (pixel, depth) sort of partials orders them for disjoint
 * domains. Replaces VolumeRenderer::DoExecute with
 * RenderOneDomainPerRank / RenderMultipleDomainsPerRank, the partial
 * extraction, PartialCompositor::composite and partials_to_canvas
 * (VolumeRenderer.cpp:141-391, 469-597; PartialCompositor.cpp:57-90,
 * 244-547). `samples_out` (may be NULL) receives the number of samples the
 * march evaluated. */
GVR_API int gvr_render_volume(gvr_scene *scene, const gvr_camera *camera,
                      const gvr_render_params *params, float *rgba,
                      float *depth, int out_location, void *stream,
                      uint64_t *samples_out);

/* Render the volume over an opaque canvas: rgba and depth (in `location`
 * memory) hold on entry the colours and image-space depths (0.5 z_ndc + 0.5,
 * 1 = nothing drawn) that the scene's opaque plots left, and on return the
 * canvas with the volume composited in front. Each ray stops where the
 * canvas depth unprojects to (the ray's MaxDistance after
 * RayOperations::MapCanvasToRays, VolumeRenderer.cpp:243-247); partials
 * blend over the canvas colour as partials_to_canvas does
 * (VolumeRenderer.cpp:366-385); pixels no partial reaches keep the canvas.
 * This is the volume pass of a mixed scene after vtkh::Scene::Render's
 * opaque pass (Scene.cpp:154-212). */
GVR_API int gvr_render_volume_over(gvr_scene *scene, const gvr_camera *camera,
                                   const gvr_render_params *params, float *rgba, float *depth,
                                   int location, void *stream, uint64_t *samples_out);

/* Render n_views cameras of the scene in one persistent launch: rgba holds
 * n_views images of 4*W*H floats and depth n_views images of W*H floats,
 * view-major, each image exactly what gvr_render_volume returns for that
 * camera. A device work queue hands out (view, tile) items; each 16x16 tile
 * marches only the domains whose projected bounds touch it. The counter
 * reset and the launch are captured as a CUDA graph, rebuilt only when the
 * launch configuration (parameters, view count, buffers, launch shape)
 * changes. Replaces the per-view loop of vtkh::Scene::Render over Cinema
 * cameras (Scene.cpp:124-247, ascent_runtime_rendering_filters.cpp:906-960).
 * With stream NULL the call uses a scene-owned stream and waits for it. */
GVR_API int gvr_render_volume_batch(gvr_scene *scene, const gvr_camera *cameras, int n_views,
                                    const gvr_render_params *params, float *rgba,
                                    float *depth, int out_location, void *stream,
                                    uint64_t *samples_out);

/* Work-queue granularity of the batch path: 16x16 tiles per item (1..64);
 * set by the autotuner. No counterpart in the reference. */
GVR_API int gvr_scene_set_batch_granularity(gvr_scene *scene, int tiles_per_item);

/* Number of CUDA graphs the batch path has captured for this scene (a
 * diagnostic; no counterpart in the reference). */
GVR_API int gvr_scene_batch_graph_builds(const gvr_scene *scene, int *n);

/* ------------------------------------------------------------------ */
/* Differentiable render (no counterpart in the reference)              */
/* ------------------------------------------------------------------ */

/* Floats per ray of the training workspace the differentiable forward
 * fills for a grid of node dims and spacing at this sample distance: one
 * transmittance checkpoint every 64 samples plus the scalar of every sample.
 * The workspace holds n_views * W * H * floats_per_ray floats. */
GVR_API int gvr_diff_workspace(const int dims[3], const double spacing[3], float sample_dist,
                               int *floats_per_ray);

/* Forward render of one uniform domain for 1..64 views with a linearly
 * interpolated transfer function and no partial culling, so that the image
 * is differentiable in the node field and the LUT. field (node values, x
 * fastest), lut (lut_size RGBA floats), rgba (n_views * W * H * 4) and
 * workspace (n_views * W * H * gvr_diff_workspace floats: the transmittance
 * checkpoints and per-sample scalars the adjoint needs; NULL for an
 * inference-only pass) are device pointers. Other fields of params used:
 * width, height, sample_dist, scalar range, lut_size. */
GVR_API int gvr_diff_render_forward(const float *field, const int dims[3], const double origin[3],
                                    const double spacing[3], const gvr_camera *cameras,
                                    int n_views, const gvr_render_params *params,
                                    const float *lut, float *rgba, float *workspace,
                                    void *stream);

/* Adjoint of gvr_diff_render_forward: given dL/d(rgba) (device, same layout
 * as rgba) and the forward's workspace, ADD dL/d(field) into grad_field
 * (node layout) and dL/d(lut) into grad_lut (lut_size * 4). The
 * transmittances of each 64-sample segment are rebuilt from its checkpoint;
 * the blend is never inverted. Scratch (a float4 per node for the
 * field-gradient corner quads, and LUT-gradient copies of at most 512 MB)
 * comes from the library's stream-ordered memory pool, which keeps the
 * memory it has handed out (up to its high-water mark) until the process
 * exits, so repeated calls map no new pages. */
GVR_API int gvr_diff_render_backward(const float *field, const int dims[3],
                                     const double origin[3], const double spacing[3],
                                     const gvr_camera *cameras, int n_views,
                                     const gvr_render_params *params, const float *lut,
                                     const float *grad_rgba, const float *workspace,
                                     float *grad_field, float *grad_lut, void *stream);

/* One ray segment's composited colour: the record of VolumePartial<float>
 * (vtkh/compositing/VolumePartial.hpp:13-20), 24 bytes. rgb is
 * premultiplied by alpha; depth orders the partials of one pixel. */
typedef struct {
  int32_t pixel_id;
  float depth;
  float rgb[3];
  float alpha;
} gvr_partial;

/* Composite partials into one record per pixel. Replaces
 * PartialCompositor<VolumePartial<float>>::composite
 * (vtkh/compositing/PartialCompositor.cpp:494-547: merge :244-325, then
 * composite_partials :331-490 and BlendPartials :57-90) for the partials of
 * all images laid end to end in `partials` (n records).
 *
 * Records are ordered by (pixel_id, depth) — records with equal keys keep
 * their input order — and each pixel's records are blended front to back
 * with VolumePartial::blend (VolumePartial.hpp:53-62), keeping the front
 * record's depth. Output order is the reference's: pixels with a single
 * record first, then blended pixels, each group in pixel order. `out`
 * needs room for n records and must not overlap `partials`; *n_out
 * receives the count. Blend arithmetic is
 * FP32 with no fused multiply-add, so results equal the reference compiled
 * without contraction bit for bit.
 *
 * location says where both `partials` and `out` live (GVR_MEM_HOST or
 * GVR_MEM_DEVICE); n < 2^31. Scratch comes from the library's
 * stream-ordered memory pool (kept between calls, as for the adjoint): 8
 * bytes per record plus 16 per pixel of the id range (dense ids) or 40 per
 * record (sparse ids), and 48 per record more for host arrays. The call
 * returns after the result is complete. */
GVR_API int gvr_composite_partials(const gvr_partial *partials, int64_t n, gvr_partial *out,
                                   int64_t *n_out, int location, void *stream);

/* Convert a float canvas (width x height RGBA, row 0 at the bottom, the
 * layout gvr_render_volume writes) into the 8-bit rows of its PNG: rows
 * flipped so that row 0 is the top one, each channel
 * (unsigned char)(value * 255) after clamping to [0, 255] — the pixel loop
 * of PNGEncoder::Encode(const float *) (png_utils/ascent_png_encoder.cpp:
 * 77-118), run on the device. `out` holds width * height * 4 bytes.
 * location says where both buffers live; with GVR_MEM_HOST the call copies
 * in and out and returns when `out` is written, with GVR_MEM_DEVICE it is
 * stream-ordered on `stream`. */
GVR_API int gvr_canvas_to_rgba8(const float *rgba, int width, int height, uint8_t *out,
                                int location, void *stream);

/* Draw the body of a colour bar into a float canvas (width x height, RGBA,
 * row 0 at the bottom): the pixels of `box` = {xmin, xmax, ymin, ymax} in
 * screen coordinates [-1, 1] (clipped to the image) take the colour-table
 * entry of their position along the box's long axis (vertical when the box
 * is taller than wide, low values at the bottom / left), opaque; the
 * rectangle's outermost pixels take `fg`. This is the coloured part of the
 * bars Render::RenderScreenAnnotations draws for each plot's colour table
 * (vtkh/rendering/Render.cpp:205-227, positions of Annotator.cpp:15-24, or
 * the render's `color_bar_position`); the tick marks, labels and field name
 * the reference draws with VTK-m's text rendering are not drawn. lut_rgba
 * is a host array of lut_size RGBA entries (2 .. 4096); the canvas lives
 * where `location` says. Returns when the bar is drawn. */
GVR_API int gvr_canvas_color_bar(float *rgba, int width, int height, const float *lut_rgba,
                                 int lut_size, const float box[4], const float fg[4],
                                 int location, void *stream);

/* gvr_composite_partials for device records whose pixel ids the caller
 * bounds, without any host synchronisation; no counterpart in the
 * reference (its composite is host code). Every record's pixel_id must lie
 * in [pixel_lo, pixel_hi] — for partials of a W x H image, [0, W H - 1] —
 * so the pixel-id range need not be measured and read back, and the output
 * count is written to *n_out, a device int64, instead of being returned:
 * the whole call is stream-ordered on `stream`. partials, out and n_out are
 * device pointers; out needs room for n records. Same order and blend as
 * gvr_composite_partials, bit for bit. A record outside the range is left
 * out and *n_out becomes -1. Scratch: 16 bytes per pixel of the range plus
 * 8 per record, from the library's pool. */
GVR_API int gvr_composite_partials_async(const gvr_partial *partials, int64_t n,
                                         int32_t pixel_lo, int32_t pixel_hi, gvr_partial *out,
                                         int64_t *n_out, void *stream);

/* Z-buffer compositing of n_images opaque canvases of width x height
 * pixels (RGBA float, row-major, + depth float): Renderer::Composite in
 * Z_BUFFER_SURFACE mode, which composites the per-domain (or per-plot)
 * renders of the opaque plots before the volume pass draws over them
 * (vtkh/rendering/Renderer.cpp:111-142; Compositor::AddImage,
 * vtkh/compositing/Compositor.cpp:86-125; ImageCompositor::ZBufferComposite,
 * ImageCompositor.hpp:49-76). Each canvas goes through the 8-bit vtkh::Image
 * (channel = (unsigned char)(value * 255), depth = |depth|, Image.hpp:80-113);
 * image 0 is kept, and image k > 0 replaces a pixel where its depth is <= 1
 * and not behind the kept depth; the result comes back as value / 255 with
 * the kept depth (Renderer::ImageToCanvas, Renderer.cpp:271-289). The output
 * is what gvr_render_volume_over takes as its opaque canvas (Scene.cpp:
 * 154-212). rgba[k] / depth[k] point at the canvases (4 W H and W H floats),
 * all on the side `location` names; n_images 1 .. 64. With GVR_MEM_HOST the
 * call stages the canvases through pooled scratch and returns when the output
 * is written; with GVR_MEM_DEVICE it is stream-ordered on `stream`. */
GVR_API int gvr_zbuffer_composite(int n_images, const float *const *rgba,
                                  const float *const *depth, int width, int height,
                                  float *out_rgba, float *out_depth, int location, void *stream);

/* Give the library's scratch memory on `device` back to the system down to
 * keep_bytes (0: everything not in use); no counterpart in the reference.
 * The partial compositor, the adjoint and the device PNG conversion take
 * their scratch from a stream-ordered pool of this library that keeps its
 * blocks between calls (its footprint grows to the largest call's scratch
 * and stays reserved until the process exits or this call trims it), so
 * that repeated calls neither map fresh pages nor synchronise. An in-situ
 * host that needs the memory back between visualisation steps calls this;
 * the next call that needs scratch allocates it again. reserved_out (may be
 * NULL) receives the bytes the pool still reserves. Synchronise the streams
 * that used the library before trimming, or their last frees may not have
 * completed yet. */
GVR_API int gvr_scratch_trim(int device, uint64_t keep_bytes, uint64_t *reserved_out);

/* Render one uniform domain without allocating any device memory; no
 * counterpart in the reference. For callers that may not call cudaMalloc or
 * cudaFree — typically a simulation that gives all GPU memory to its own
 * pool allocator, where a library allocation can fail against the pool's
 * budget and cudaMalloc/cudaFree would synchronise the device under the
 * simulation's streams.
 *
 * `field` is a device pointer to dims[0]*dims[1]*dims[2] float32 node values
 * (x fastest); `rgba` (4*W*H floats) and `depth` (W*H floats) are device
 * pointers; all must live on the calling thread's current CUDA device. The
 * result equals gvr_render_volume on a scene holding this one domain.
 * `samples_out` (may be NULL) is a host pointer; when given, the call waits
 * for the render to finish.
 *
 * Scratch: the device copy of the LUT and the sample counter live in one
 * fixed 64 KiB + 256 B array inside the library, which every GPU that loads
 * the library holds until the process exits. lut_size above 4096 is
 * rejected. The first call on a device looks up that array's device address
 * (set-up), so make the first call on each device before any stream
 * capture. Every call shares the array: calls that overlap on the GPU race
 * on it, so serialise them (one stream, or wait between calls). */
GVR_API int gvr_render_uniform_noalloc(const float *field, const int dims[3],
                                       const double origin[3], const double spacing[3],
                                       const gvr_camera *camera,
                                       const gvr_render_params *params, float *rgba,
                                       float *depth, void *stream, uint64_t *samples_out);

#ifdef __cplusplus
}
#endif

#endif /* GVR_H */
