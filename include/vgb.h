/*
 * vgb.h - C ABI of the GB300 spectral ray-tracing hot path (vira_gb300).
 *
 * This is the drop-in boundary for Vira's CPU path tracer.  The reference is a
 * header-only C++ template library with two seams on this path:
 *
 *   (1) the renderer object   CPUPathTracer::render(Camera&, Scene&), its public
 *       `options` and `renderPasses` (include/vira/rendering/cpu_path_tracer.hpp:46-58),
 *       called from Scene::pathtraceRender / renderTotalPower
 *       (include/implementation/scene.ipp:840-915);
 *   (2) the acceleration plugin  TLAS::intersect(Ray&) / BLAS::intersect
 *       (include/vira/rendering/acceleration/tlas.hpp:20-31, blas.hpp:20-37), which
 *       Embree fills through rtcIntersect1
 *       (include/implementation/rendering/acceleration/embree_tlas.ipp:128-173).
 *
 * Every entry point returns a vgb_status and never throws or aborts (a failed host
 * allocation inside a call returns VGB_ERR_OUT_OF_MEMORY).  Buffers are
 * owned by the caller unless a vgb_*_create function made them.  A context owns one
 * CUDA stream and is not thread-safe: use one host thread per context.
 *
 * Conventions
 *   - B = number of spectral bands (1..VGB_MAX_BANDS).
 *   - Images are planar, row-major: plane[b][j][i] at b*W*H + j*W + i, which is the
 *     reference's linear index i + j*W (include/implementation/images/image.ipp:137)
 *     with the bands split into planes.
 *   - Matrices are column-major like glm: m[c*rows + r].
 *   - Triangle ids are the index of the triangle in the caller's index buffer.
 */
#ifndef VGB_H
#define VGB_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#if defined(_WIN32)
#define VGB_API __declspec(dllexport)
#else
#define VGB_API __attribute__((visibility("default")))
#endif

#define VGB_MAX_BANDS 8
#define VGB_NO_HIT 0xFFFFFFFFu

typedef enum vgb_status {
    VGB_OK = 0,
    VGB_ERR_INVALID_ARGUMENT = 1, /* bad pointer, size or option (reference: std::runtime_error) */
    VGB_ERR_CUDA = 2,             /* a CUDA runtime call failed */
    VGB_ERR_OUT_OF_MEMORY = 3,    /* device or host allocation failed */
    VGB_ERR_NOT_READY = 4,        /* no scene uploaded / no BVH built yet */
    VGB_ERR_DEVICE_LIMIT = 5,     /* a kernel hit its traversal-stack or iteration cap */
    VGB_ERR_INTERNAL = 6
} vgb_status;

typedef struct vgb_context vgb_context;

/* ---- camera: FP32 constants derived on the host in FP64 -------------------------
 * Replaces Camera::pixelToRay (include/implementation/cameras/camera.ipp:1126-1131,
 * 1143-1163), pixelToDirection / pixelToDirectionHelper (:1105-1117, 1738-1749) and
 * ReferenceFrame::localDirectionToGlobal (include/implementation/reference_frame.ipp:361-364).
 * The ray of pixel coordinate (x, y) is
 *     h     = kinv·(x, y, 1), then h = undistort(h) when a distortion model is set
 *     d_cam = { h[0],  z_dir * h[1],  z_dir }
 *     dir   = normalize(rotation · d_cam),   origin = origin.
 * With a distortion and interpolate_directions (the reference's default), d_cam is instead the
 * bilinear interpolation (Image::interpolatePixel) of normalize(d_cam) at the four surrounding
 * integer pixels, as Camera::precomputePixelDirections (:1676-1700) tabulates it.
 * Depth of field (samples >= 1 only, as the reference's sample 0 goes through the pinhole
 * overload): a point a of the circular aperture (radius * UniformDiskSample) moves the origin by
 * rotation · (a.x, a.y, focal_length), and with a finite focus distance the camera direction
 * becomes focus_distance * normalize(d_cam) - (a.x, a.y, focal_length). */
typedef enum vgb_distortion_model {
    VGB_DISTORTION_NONE = 0,
    VGB_DISTORTION_BROWN = 1,   /* coeffs: k1 k2 k3 p1 p2 (brown_distortion.ipp) */
    VGB_DISTORTION_OPENCV = 2,  /* coeffs: k1 k2 k3 k4 k5 k6 p1 p2 s1 s2 s3 s4 (opencv_distortion.ipp) */
    VGB_DISTORTION_OWEN = 3     /* coeffs: e1 e2 e3 e4 e5 e6 (owen_distortion.ipp) */
} vgb_distortion_model;

typedef struct vgb_camera {
    uint32_t width;            /* resolution x (columns, index i) */
    uint32_t height;           /* resolution y (rows, index j) */
    float origin[3];           /* camera position in the scene frame (rebased in FP64, then FP32) */
    float rotation[9];         /* camera-to-scene rotation, column-major 3x3 */
    float kinv[6];             /* inverse intrinsic matrix, column-major 3 columns x 2 rows */
    float z_dir;               /* +1, or -1 for the Blender frame */
    float power_scale[VGB_MAX_BANDS]; /* optical efficiency[b] * aperture area (received power) */
    /* lens distortion (Camera::setBrownDistortion / setOpenCVDistortion / setOwenDistortion):
     * undistorted by 20 fixed-point iterations in FP32 for rays and the pixel solid angle,
     * distorted in the rasterizer's projection (Camera::projectCameraPoint, camera.ipp:1060-1080) */
    uint32_t distortion;       /* vgb_distortion_model */
    float distortion_coeffs[12];
    uint32_t interpolate_directions; /* Camera::interpolate_distortion_directions_ (default 1) */
    /* depth of field (Camera::enableDepthOfField, setFocusDistance, CircularAperture) */
    uint32_t depth_of_field;   /* 0: pinhole for every sample (reference default) */
    float aperture_radius;     /* focal_length / f_stop / 2 (metres) */
    float focal_length;        /* metres */
    float focus_distance;      /* metres; +inf keeps the pinhole direction (reference default) */
    /* first-hit passes (cpu_path_tracer.ipp:356-372): Camera::calculateGSD's sensor size and the
     * camera's motion.  The reference evaluates the camera's point velocity at the hit point's
     * global coordinates taken as if they were camera-local (localPointToGlobalVelocity on
     * intersection_global), i.e. at rotation * p_global; rot_origin = rotation * (scene origin),
     * FP64 then FP32, restores that term in the rebased frame: rotation * p + rot_origin. */
    float sensor_size[2];      /* metres */
    float velocity[3];         /* global frame, m/s */
    float angular_rate[3];     /* global frame, rad/s */
    float rot_origin[3];
} vgb_camera;

/* ---- sphere light (Vira's SphereLight; the Sun is one) --------------------------
 * include/implementation/lights/sphere_light.ipp:17-153. */
typedef struct vgb_light {
    float position[3];         /* centre in the scene frame (FP64 ephemeris, rebased, FP32) */
    float radius;              /* metres */
    float radiance[VGB_MAX_BANDS]; /* spectral radiance per band */
} vgb_light;

/* ---- path tracer options: CPUPathTracerOptions + RenderPasses switches ----------
 * include/vira/rendering/cpu_path_tracer.hpp:30-43, include/vira/rendering/passes.hpp:72-84. */
/* ---- EATWT denoiser options (rendering/cpu_denoise.hpp:10-19, EATWTOptions) ---------- */
typedef struct vgb_denoise_options {
    uint32_t levels_direct;      /* MAX_LEVELS_DIRECT (5) */
    uint32_t levels_indirect;    /* MAX_LEVELS_INDIRECT (5) */
    float depth_threshold;       /* DEPTH_THRESHOLD (0.2) */
    float normal_threshold;      /* NORMAL_THRESHOLD (0.5) */
    float min_normal_weight;     /* MIN_NORMAL_WEIGHT (0.3) */
    float epsilon;               /* EPSILON (1e-6) */
} vgb_denoise_options;

typedef struct vgb_pt_options {
    uint32_t samples;            /* options.samples (>= 1) */
    uint32_t bounces;            /* options.bounces */
    uint32_t show_background;    /* options.show_background (uniform background emission) */
    uint32_t simulate_lighting;  /* renderPasses.simulate_lighting */
    uint32_t smooth_shading;     /* Mesh::getSmoothShading */
    uint32_t deterministic_light;/* 1: RNG-free SphereLight::sample (sphere_light.ipp:31-64) */
    uint32_t rr_depth;           /* Russian roulette from this bounce on; 0 = off (reference) */
    uint32_t has_ambient;        /* Scene::hasAmbient */
    uint64_t seed;               /* counter-based RNG key */
    uint32_t frame;              /* counter-based RNG key, second word */
    uint32_t nbands;             /* B */
    float ambient[VGB_MAX_BANDS];
    float background[VGB_MAX_BANDS];
    /* adaptive sampling (cpu_path_tracer.ipp:198-226): after sample s (s > 0), a pixel stops
     * when s is a multiple of samples_to_detect_miss and no sample has hit yet, or s is a
     * multiple of samples_per_batch and the 95% interval of the path-radiance magnitude is within
     * sampling_tolerance of its mean (or every magnitude was 0); the pixel's planes are then
     * divided by s, as the reference does.  0 = off (reference default). */
    uint32_t adaptive_sampling;
    uint32_t samples_per_batch;      /* options.samples_per_batch (reference default 30) */
    float sampling_tolerance;        /* options.sampling_tolerance (reference default 0.05) */
    uint32_t samples_to_detect_miss; /* options.samples_to_detect_miss (reference default 30) */
    /* options.denoise (cpu_path_tracer.ipp:124-134): after the samples, the direct and indirect
     * radiance are filtered by the edge-avoiding a-trous wavelet transform guided by albedo,
     * depth and normal, the total radiance becomes their sum and the received power follows
     * from it.  0 = off (reference default). */
    uint32_t denoise;
    vgb_denoise_options denoiser;    /* zero-filled: the reference's EATWTOptions defaults */
} vgb_pt_options;

/* ---- film: RenderPasses planes (caller-owned; NULL = pass not written) ----------
 * include/vira/rendering/passes.hpp:51-95, passes.ipp:43-128. */
typedef struct vgb_film {
    float* total_radiance;     /* [B][H][W] */
    float* direct_radiance;    /* [B][H][W] */
    float* indirect_radiance;  /* [B][H][W] */
    float* received_power;     /* [B][H][W]; needs pixel_solid_angle */
    float* albedo;             /* [B][H][W] */
    float* normal_global;      /* [3][H][W] */
    float* depth;              /* [H][W]; +inf where nothing was hit */
    float* alpha;              /* [H][W] */
    uint32_t* triangle_id;     /* [H][W]; VGB_NO_HIT where nothing was hit */
    const float* pixel_solid_angle; /* [H][W] input, from vgb_pixel_solid_angle */
    int32_t on_device;         /* 1: every pointer is device memory; 0: host memory (vgb_render:
                                  pinned planes, cudaHostAlloc or cudaHostRegister, are written by
                                  the kernels through their mapped address; pageable ones are
                                  staged in device memory and copied back) */
    /* renderPasses.save_velocity / save_triangle_size (passes.hpp:79-85), set at a pixel's first
     * hit (cpu_path_tracer.ipp:356-372); pixels that never hit keep 0 / +inf */
    float* velocity_global;    /* [3][H][W] the hit point's velocity (instance motion) */
    float* velocity_camera;    /* [3][H][W] relative to the camera, in the camera frame */
    float* triangle_size;      /* [H][W] longest edge of the hit triangle / GSD at the hit distance */
} vgb_film;

/* ---- BVH build options -------------------------------------------------------- */
typedef struct vgb_bvh_options {
    uint32_t max_leaf_size;    /* triangles per leaf: 1..8 (binary), 1..3 (8-wide); 0 = default */
    uint32_t builder;          /* 0 = binned SAH (host, threaded); 1 = linear BVH on the GPU (30-bit Morton
                                  order, Karras's hierarchy, ranges of <= max_leaf_size triangles as leaves;
                                  binary layout only; seconds -> milliseconds at tens of millions of
                                  triangles, at some traversal speed) */
    uint32_t threads;          /* host threads for the build; 0 = all */
    uint32_t layout;           /* device node layout: 2 = binary (default, 0), 8 = compressed 8-wide */
} vgb_bvh_options;

/* ---- statistics of the last render / trace ------------------------------------ */
typedef struct vgb_stats {
    uint64_t rays_closest;     /* closest-hit queries (primary + bounce) */
    uint64_t rays_shadow;      /* shadow (any-hit) queries */
    uint64_t nodes_visited;    /* counting pass only: wide nodes visited, all queries */
    uint64_t tris_tested;      /* counting pass only: triangle records tested, all queries */
    uint64_t nodes_closest;    /* counting pass only: nodes visited by closest-hit queries */
    uint64_t tris_closest;     /* counting pass only: triangles tested by closest-hit queries */
    uint64_t hits_closest;     /* closest-hit queries that hit (shaded) */
    uint32_t bvh_nodes;        /* nodes in the device BVH */
    uint32_t bvh_node_bytes;   /* bytes per node */
    uint32_t tri_record_bytes; /* bytes per triangle record */
    uint32_t kernel_launches;  /* kernels launched by the last render */
    uint32_t device_error;     /* last device error word (0 = none) */
    float ms_last;             /* device time of the last render, or of the device phase of the last vgb_quipu_read_mesh (CUDA events) */
    /* profiling mode only (vgb_set_profiling): device time and launches per kernel family:
     * closest-hit traversal, shading, shadow traversal, film */
    float ms_trace, ms_shade, ms_shadow, ms_film;
    uint32_t launches_trace, launches_shade, launches_shadow, launches_film;
} vgb_stats;

/* ========================= context ============================================= */
VGB_API vgb_status vgb_context_create(vgb_context** out, int device);
VGB_API vgb_status vgb_context_destroy(vgb_context* ctx);
VGB_API const char* vgb_last_error(const vgb_context* ctx);
VGB_API const char* vgb_version(void);
/* Make the context use an existing CUDA stream (cudaStream_t passed as void*); NULL = own. */
VGB_API vgb_status vgb_set_stream(vgb_context* ctx, void* stream);
VGB_API vgb_status vgb_synchronize(vgb_context* ctx);

/* ========================= host-side geometry ================================== */
/* Mesh::calculateNormals (include/implementation/geometry/mesh.ipp:199-233): each vertex
 * normal is the sum, in triangle order, of the unit face normals normalize(cross(p1-p0,
 * p2-p0)) of its triangles (NaN face normals skipped), then normalised.  Host C++. */
VGB_API vgb_status vgb_compute_vertex_normals(const float* positions, uint32_t nverts,
                                              const uint32_t* indices, uint32_t ntris,
                                              float* normals_out);
/* DEM::makeVertexBuffer (include/implementation/dems/dem.ipp:165-211) with the non-OGR grid
 * mapping (include/implementation/dems/dem_projection.ipp:131-141) and imageToIndexBuffer
 * (include/implementation/images/image_utils.ipp:364-409).  heights: [H][W] row-major.
 * positions_out: 3*W*H floats; indices_out: up to 6*(W-1)*(H-1); *ntris_out = count. */
VGB_API vgb_status vgb_dem_triangulate(const float* heights, uint32_t width, uint32_t height,
                                       double posting_x, double posting_y,
                                       float* positions_out, uint32_t* indices_out,
                                       uint32_t* ntris_out);
/* Camera::initializeIntrinsicMatrix (include/implementation/cameras/camera.ipp:1526-1568),
 * evaluated in FP32 as the reference's TFloat = float instantiation does.
 * px/py = +inf selects the image centre. */
VGB_API vgb_status vgb_camera_intrinsics(float focal_length, float sensor_x, float sensor_y,
                                         uint32_t width, uint32_t height, float px, float py,
                                         float kxy, float kyx, float z_dir, float kinv_out[6]);

/* ========================= scene / BVH ========================================= */
/* Scene::buildTLAS input (include/implementation/scene.ipp:712-812): one flattened triangle
 * mesh in the scene frame.  vert_albedo: B floats per vertex or NULL (=1);
 * vert_normal: 3 floats per vertex or NULL (computed); vert_uv: 2 floats per vertex or NULL
 * (=0); texture: albedo map [tex_h][tex_w][B] or NULL (1x1 of 1.0, material.hpp:72).
 * Host pointers.  Uploading replaces the scene and invalidates the BVH. */
VGB_API vgb_status vgb_scene_upload(vgb_context* ctx, const float* positions, uint32_t nverts,
                                    const uint32_t* indices, uint32_t ntris, uint32_t nbands,
                                    const float* vert_albedo, const float* vert_normal,
                                    const float* vert_uv, const float* texture,
                                    uint32_t tex_w, uint32_t tex_h);
/* Instance motion for the first-hit velocity pass (ReferenceFrame::localPointToGlobalVelocity,
 * reference_frame.ipp:367-373): velocity = v + angular_rate x (p - position) for the triangles
 * [first_triangle, next instance's first_triangle) of the uploaded (flattened) mesh. */
typedef struct vgb_instance_motion {
    uint32_t first_triangle;   /* ascending over the table, the first entry 0 */
    float velocity[3];         /* global frame, m/s */
    float angular_rate[3];     /* global frame, rad/s */
    float position[3];         /* the instance's origin in the scene frame (rebased FP64, then FP32) */
} vgb_instance_motion;

/* Replaces the motion table of the uploaded scene (host pointer; n = 0 or NULL: every instance at
 * rest).  Set it after vgb_scene_upload, which clears it. */
VGB_API vgb_status vgb_scene_motion(vgb_context* ctx, const vgb_instance_motion* motion, uint32_t n);

/* Material::setNormalMap / getNormal (include/implementation/materials/material.ipp:120-143,
 * cpu_path_tracer.ipp:316-329): a tangent-space normal map [h][w][3] (host pointer) for the
 * uploaded scene, sampled like the albedo texture (wrap + bilinear at uv * resolution); at a hit
 * the shading normal becomes normalize([tangent | bitangent | N] * sample), used by next-event
 * estimation, MIS, the film's normal and the rasterizer, while the continuation direction is
 * still sampled in the frame built before the map (the reference's order).  NULL (or w or h 0)
 * removes the map.  Set it after vgb_scene_upload, which clears it.  The adjoint entry points
 * reject a scene with a normal map (its derivative is not formed). */
VGB_API vgb_status vgb_scene_normal_map(vgb_context* ctx, const float* normal_map, uint32_t w, uint32_t h);
/* Replaces Mesh::buildBVH -> EmbreeBLAS (include/implementation/geometry/mesh.ipp:396-408,
 * include/implementation/rendering/acceleration/embree_blas.ipp:14-71). */
VGB_API vgb_status vgb_bvh_build(vgb_context* ctx, const vgb_bvh_options* opts);
/* Moves the uploaded vertices (same triangles), in place of re-uploading the mesh and rebuilding
 * the BVH that Scene::buildTLAS does when geometry changed (include/implementation/scene.ipp:711-805).
 * positions: 3 floats per vertex; normals: 3 floats per vertex or NULL (recomputed on the device,
 * the same normals vgb_compute_vertex_normals gives); both device memory if on_device else host.
 * A binary BVH is refitted on the device (every box recomputed bottom up, topology kept: the
 * boxes equal a rebuild's for unchanged positions); an 8-wide BVH is rebuilt. */
VGB_API vgb_status vgb_scene_update_positions(vgb_context* ctx, const float* positions, const float* normals,
                                              int on_device);

/* ========================= rendering =========================================== */
/* Camera::initializePixelSolidAngle (include/implementation/cameras/camera.ipp:1622-1666):
 * Girard's theorem on the four corner directions, FP64, one device kernel.
 * out: [H][W] floats, device memory if out_on_device else host. */
VGB_API vgb_status vgb_pixel_solid_angle(vgb_context* ctx, const vgb_camera* cam, float* out,
                                         int out_on_device);
/* CPUPathTracer::render (include/implementation/rendering/cpu_path_tracer.ipp:29-161). */
VGB_API vgb_status vgb_render(vgb_context* ctx, const vgb_camera* cam, const vgb_light* lights,
                              uint32_t nlights, const vgb_pt_options* opts, vgb_film* film);
/* Render without allocating.  No counterpart in the reference: Vira's CPU tracer has no
 * device memory to manage.  For callers that cannot allocate device memory once their scene is
 * set up -- a frame loop held to a fixed memory budget, or a host application whose own
 * allocator owns the device -- because a cudaMalloc inside a render call can synchronize the
 * device or fail.  Same launch sequence, kernels and results as vgb_render (bit for bit), with
 * every byte of scratch taken from one fixed 8 MiB array compiled into the library, which every
 * GPU that loads the library holds until the process exits.  Limits: the film must be device
 * memory; a frame of P = width*height pixels (T = its pixels rounded up to whole 8x4 tiles),
 * B bands and L lights needs about 4 * (P * (15 + 6*B + L*(8 + B)) + 4*T) bytes of the 8 MiB
 * (about 25,000 pixels at 8 bands and 1 light, 38,000 at 4 bands); larger frames are rejected
 * with VGB_ERR_INVALID_ARGUMENT and a message naming the sizes, as are frames past vgb_render's
 * limits; adaptive sampling and denoising are refused.  The first call on a context looks up
 * the array's device address (cudaGetSymbolAddress) with the context's device current: make
 * that first call before any stream capture.  The first call for a band count (1, 2-4, 5-8)
 * and BVH layout may load those kernels' code onto the device under CUDA's lazy module loading
 * (CUDA_MODULE_LOADING=EAGER loads them all at start-up).  Each call waits for ctx's stream
 * and copies the device error word and ray counts to the host before it returns, as vgb_render
 * does, so no call may be made while ctx's stream is being captured into a CUDA graph.  The
 * context keeps the array's address; like every other device object of the context it does not
 * survive a cudaDeviceReset (destroy the context first).  vgb_get_stats then reports the rays, launches and device time of this call and zeros
 * for the counting-pass and profiling fields, which this entry point does not fill.  All calls
 * on a device share the array and it keeps the last call's contents (each call clears its
 * counters itself): calls that overlap on the GPU -- two contexts or two streams rendering at
 * once on one device -- race. */
VGB_API vgb_status vgb_render_noalloc(vgb_context* ctx, const vgb_camera* cam, const vgb_light* lights,
                                      uint32_t nlights, const vgb_pt_options* opts, vgb_film* film);
/* ---- batched trajectory rendering -------------------------------------------------
 * Many frames (cameras, lights, resolutions and sample counts of their own) rendered by one
 * persistent kernel: warps claim (frame, 8x4-pixel tile) items from a queue, the most expensive
 * frames first, and keep each tile's samples in registers and shared memory.  Per-pixel results
 * are those of vgb_render for the same frame (same arithmetic and random streams).  No
 * counterpart in the reference, which renders one frame per call. */
typedef struct vgb_frame {
    vgb_camera camera;
    vgb_light lights[8];
    uint32_t nlights;
    uint32_t samples;          /* this frame's samples per pixel */
    uint32_t frame;            /* RNG key word of this frame (vgb_pt_options.frame for vgb_render) */
    vgb_film film;             /* device planes (on_device must be 1) */
} vgb_frame;

typedef struct vgb_batch_options {
    uint32_t autotune;         /* 1: time launch shapes on a 1/16 sample of the tiles, keep the best */
    uint32_t use_graph;        /* 1: replay the batch from a captured CUDA graph */
    uint32_t block_threads;    /* 0: default or tuned (64, 128 or 256) */
    uint32_t blocks_per_sm;    /* 0: default or tuned */
    uint32_t tiles_per_grab;   /* work items claimed per queue access; 0: default or tuned */
} vgb_batch_options;

/* Renders `nframes` frames with the options in `opts` (samples and frame are taken from each
 * vgb_frame).  Frames' film planes are written as by vgb_render. */
VGB_API vgb_status vgb_render_batch(vgb_context* ctx, const vgb_frame* frames, uint32_t nframes,
                                    const vgb_pt_options* opts, const vgb_batch_options* bopts);
/* The launch shape chosen by the last autotuned batch (0s before the first one). */
VGB_API vgb_status vgb_batch_tuning(vgb_context* ctx, uint32_t* block_threads, uint32_t* blocks_per_sm,
                                    uint32_t* tiles_per_grab);

/* ---- adjoint (differentiable rendering; no counterpart in the reference) -------------
 * Given dL/dI for the total-radiance planes ([B][H][W]) of a frame rendered with the same
 * camera, lights and options, ADDS into d_texture ([tex_h][tex_w][B], the albedo texture's
 * layout) and d_height (one per vertex: the derivative with respect to the vertex's z in the
 * scene frame); NULL skips one.  Paths are replayed from their random streams, nothing is stored
 * by the forward render.  Height gradients go through the shading normal in every next-event
 * term (flat shading: the hit triangle's face normal; smooth shading: the interpolated vertex
 * normals, see vgb_adjoint_positions) and through the motion of the hit point on the triangle
 * (barycentrics, hence texture coordinates, interpolated albedo and interpolated normal).
 * Excluded: visibility (shadow and silhouette edges), the rotation of the sampled continuation
 * direction with the normal, the motion of the shading point, Russian roulette decisions.
 * At most 3 bounces. */
VGB_API vgb_status vgb_adjoint(vgb_context* ctx, const vgb_camera* cam, const vgb_light* lights,
                               uint32_t nlights, const vgb_pt_options* opts, const float* dL_dradiance,
                               float* d_texture, float* d_height, int on_device);
/* As vgb_adjoint, with the gradient with respect to every vertex position: ADDS into
 * d_position ([nverts][3], scene frame).  With smooth shading the shading normal's gradient goes
 * back through the vertex normals of each hit triangle to the positions of their 1-rings (the
 * vertex normals must be those of vgb_compute_vertex_normals); with flat shading through the
 * face normal.  A per-vertex offset along any direction field (heights: +z; radial offsets:
 * the unit radial direction) has the gradient dot(d_position[v], direction[v]). */
VGB_API vgb_status vgb_adjoint_positions(vgb_context* ctx, const vgb_camera* cam, const vgb_light* lights,
                                         uint32_t nlights, const vgb_pt_options* opts,
                                         const float* dL_dradiance, float* d_texture, float* d_position,
                                         int on_device);

/* ---- fused forward + adjoint over many views (no counterpart in the reference) ---------
 * One persistent launch renders every view, forms the L2 loss against the view's target and
 * back-propagates it: per pixel, the samples are traced (forward), dL/dI = 2 (I - target) is
 * formed, and the same samples are replayed for the gradients.  All pointers are device memory. */
typedef struct vgb_view {
    vgb_camera camera;
    vgb_light lights[8];
    uint32_t nlights;
    uint32_t samples;          /* this view's samples per pixel */
    uint32_t frame;            /* RNG key word of this view */
    uint32_t pad;
    const float* target;       /* [B][H][W] */
    float* radiance;           /* [B][H][W] total radiance out (as vgb_render's), or NULL */
} vgb_view;

/* ADDS the gradients of loss = sum over views, bands and pixels of (I - target)^2 into
 * d_texture ([tex_h][tex_w][B]) and d_position ([nverts][3]) (either may be NULL) and writes the
 * loss (FP64 sum) to *loss if loss is not NULL.  The radiance planes equal vgb_render's
 * total_radiance for the same view (same arithmetic and random streams).  Exclusions as for
 * vgb_adjoint_positions; at most 3 bounces. */
VGB_API vgb_status vgb_render_adjoint_batch(vgb_context* ctx, const vgb_view* views, uint32_t nviews,
                                            const vgb_pt_options* opts, float* d_texture, float* d_position,
                                            double* loss);
/* denoiseSpectralRadianceEATWT (rendering/cpu_denoise.ipp:9-214) on caller planes: direct and
 * indirect ([B][H][W], filtered in place), albedo ([B][H][W]), depth ([H][W]) and normal_global
 * ([3][H][W]).  o may be NULL (reference defaults).  The reference indexes its images as
 * (y, x), that is transposed, so each level filters along columns first and rows second; for
 * square images this equals the reference, for other sizes the reference reads out of range and
 * this applies the same column-then-row order.  All planes device memory if on_device else host. */
VGB_API vgb_status vgb_denoise(vgb_context* ctx, float* direct, float* indirect, const float* albedo,
                               const float* depth, const float* normal, uint32_t width, uint32_t height,
                               uint32_t nbands, const vgb_denoise_options* o, int on_device);
/* ---- DEM triangulation and vertex normals on the GPU ------------------------------------
 * The same outputs as vgb_dem_triangulate and vgb_compute_vertex_normals (bit for bit): posts
 * in FP64 then FP32, the index buffer in the reference's quad order with infinite posts skipped
 * (an exclusive scan places each quad's triangles), and per-vertex sums of unit face normals in
 * face order (each vertex gathers its faces, sorted).  idx must hold 2 (W-1)(H-1) triangles;
 * *nt_out receives the count.  Arrays device memory if on_device else host. */
VGB_API vgb_status vgb_dem_triangulate_gpu(vgb_context* ctx, const float* heights, uint32_t W, uint32_t H, double sx,
                                           double sy, float* pos, uint32_t* idx, uint32_t* nt_out, int on_device);
VGB_API vgb_status vgb_compute_vertex_normals_gpu(vgb_context* ctx, const float* pos, uint32_t nverts,
                                                  const uint32_t* idx, uint32_t ntris, float* normals,
                                                  int on_device);

/* ---- sensor chain after the film ------------------------------------------------------
 * Camera::simulateSensor (cameras/camera.ipp:1218-1240): received power -> photon counts
 * (getPhotonCounts, camera.ipp:1286-1330; optional filter mosaic and Poisson photon noise) ->
 * electrons through the quantum efficiency plus the noise model's electrons (NoiseModel::simulate,
 * noise_models/noise_model.ipp:36-74: Poisson dark current x exposure time, Gaussian readout,
 * sinusoidal fixed pattern) -> gain, clamp to max ADU, normalised (Photosite::exposePixel,
 * photosites/photosite.ipp:125-136).  The reference draws from std::mt19937; here every draw
 * comes from the counter-based Philox stream keyed by (seed, frame) and the pixel, so a sensor
 * image is reproducible.  Without noise the result is deterministic and equals the reference's
 * arithmetic. */
typedef struct vgb_sensor {
    float exposure_time;              /* s (Camera default 0.01) */
    float photon_energy[8];           /* J per band, h c / centre wavelength (TSpectral::photonEnergies) */
    float quantum_efficiency[8];      /* PhotositeConfig::quantum_efficiency */
    float gain;                       /* ADU per electron (PhotositeConfig::gain) */
    float max_adu;                    /* linear_scale_factor * (2^bit_depth - 1) */
    uint32_t simulate_photon_noise;   /* Poisson photon counts where the pixel's total count >= 1 */
    uint32_t noise_model;             /* 1: NoiseModel::simulate per pixel */
    float dark_current;               /* NoiseModelConfig::dark_current */
    float readout_noise_mean;         /* NoiseModelConfig::readout_noise_mean */
    float readout_noise_std;          /* NoiseModelConfig::readout_noise_std */
    float horizontal_scale;           /* NoiseModelConfig::horizontal_scale */
    float vertical_scale;             /* NoiseModelConfig::vertical_scale */
    uint32_t horizontal_pattern_period;
    uint32_t vertical_pattern_period;
    uint32_t frame;                   /* RNG key word */
    uint64_t seed;                    /* RNG key */
    const float* filter_mosaic;       /* [B][H][W] band transmission per pixel, or NULL */
} vgb_sensor;

/* received_power [B][H][W] -> image [H][W] in 0..1.  Planes (and the mosaic) device memory if
 * on_device else host. */
VGB_API vgb_status vgb_sensor_simulate(vgb_context* ctx, const float* received_power, uint32_t width,
                                       uint32_t height, uint32_t nbands, const vgb_sensor* sensor,
                                       float* image, int on_device);
/* Camera::simulateSensorRGB (cameras/camera.ipp:1253-1282) with getPhotonCountsRGB (:1337-1380)
 * and Photosite::exposePixelRGB (photosites/photosite.ipp:145-154): each pixel's received power
 * (times the filter mosaic when one is set) is converted to ColorRGB by spectralConvert
 * (spectral_data.ipp:588-605: per RGB band the overlap-weighted sum of the spectral bands,
 * SpectralData::integrateOver, divided by the RGB bandwidth), to photons per channel (exposure /
 * ColorRGB photon energy), Poisson photon noise where the three channels hold one photon or more,
 * one NoiseModel draw per channel, then qe_rgb * photons + noise, times the gain, over max ADU --
 * with no clamp, as the reference's RGB photosite has none.  The sensor fields for the spectral
 * bands (photon_energy, quantum_efficiency) are not read. */
typedef struct vgb_rgb_conversion {
    float band_min[8];                /* the spectral bands' edges in metres (FP32, as stored) */
    float band_max[8];
    float rgb_min[3];                 /* ColorRGB's bands: R 600-750, G 500-600, B 380-500 nm, in metres */
    float rgb_max[3];
    float rgb_bandwidth[3];           /* max - min in FP32 */
    float rgb_photon_energy[3];       /* ColorRGB::photonEnergies */
    float rgb_quantum_efficiency[3];  /* PhotositeConfig::quantum_efficiency_rgb */
} vgb_rgb_conversion;

/* received_power [B][H][W] -> image_rgb [3][H][W] (R, G, B planes).  Device memory if on_device
 * else host. */
VGB_API vgb_status vgb_sensor_simulate_rgb(vgb_context* ctx, const float* received_power, uint32_t width,
                                           uint32_t height, uint32_t nbands, const vgb_sensor* sensor,
                                           const vgb_rgb_conversion* rgb, float* image_rgb, int on_device);
/* Image::convolveSpatial (images/image.ipp:1267-1340) of received_power ([B][H][W], in place)
 * with a per-band kernel ([B][kh][kw]): out(x, y) = sum over (kx, ky) of
 * in(x + kx - kw/2, y + ky - kh/2) * kernel(kx, ky), zero outside the image, rows of the kernel
 * outer.  The reference switches to an FFT for kernels of 256 or more taps (images/image.ipp:
 * 1012-1059), which equals this sum up to rounding.  Kernel sides up to 127. */
VGB_API vgb_status vgb_psf_convolve(vgb_context* ctx, float* received_power, uint32_t width, uint32_t height,
                                    uint32_t nbands, const float* kernel, uint32_t kernel_w, uint32_t kernel_h,
                                    int on_device);
/* Replaces the albedo texture (same size) without re-uploading the mesh or rebuilding the BVH. */
VGB_API vgb_status vgb_texture_update(vgb_context* ctx, const float* texture, uint32_t tex_w, uint32_t tex_h);

/* TLAS::intersect(Ray&) seam (include/vira/rendering/acceleration/tlas.hpp:24): a batch of
 * rays, closest hit (any_hit = 0) or occlusion (any_hit = 1, tmax per ray or +inf).
 * origins/dirs: 3 floats per ray.  tri_out: VGB_NO_HIT on a miss; t_out: +inf on a miss;
 * bary_out: 3 floats per ray, Interaction::w order {w(v1), w(v2), w(v0)} (ray.hpp:49,
 * embree_tlas.ipp:159-161).  tmax, t_out, bary_out may be NULL.
 * All arrays device memory if on_device else host. */
VGB_API vgb_status vgb_trace_rays(vgb_context* ctx, const float* origins, const float* dirs,
                                  const float* tmax, uint32_t nrays, int any_hit,
                                  uint32_t* tri_out, float* t_out, float* bary_out,
                                  int on_device);
/* Statistics of the last render/trace.  If count_pass is set, the next render/trace also runs
 * a counting pass that fills nodes_visited/tris_tested (algorithmic traffic). */
VGB_API vgb_status vgb_get_stats(vgb_context* ctx, vgb_stats* out);
VGB_API vgb_status vgb_set_count_pass(vgb_context* ctx, int enable);
/* Per-launch CUDA events around every kernel of vgb_render, summed per kernel family into
 * vgb_stats.ms_trace / ms_shade / ms_shadow / ms_film. */
VGB_API vgb_status vgb_set_profiling(vgb_context* ctx, int enable);
/* Read bandwidth of the GPU's L2 (a measurement utility; no counterpart in the reference): a
 * `bytes` buffer (1 MiB..16 GiB, a multiple of 16) is allocated on the context's device, read
 * once to warm the cache, then read `passes` times per launch with L2-only loads in `repeats`
 * timed launches (CUDA events on the context's stream); *gbps = the best launch's bytes read
 * per second / 1e9.  A buffer within the L2 (e.g. 64 MiB of GB300's 126 MB) measures L2, a
 * larger one HBM.  The buffer is freed before return. */
VGB_API vgb_status vgb_measure_l2_read(vgb_context* ctx, uint64_t bytes, uint32_t passes, uint32_t repeats,
                                       double* gbps);
/* How vgb_render and vgb_render_noalloc traverse the binary BVH (no counterpart in the
 * reference; results do not depend on it).  persistent = 0 (default): one thread per ray in
 * grid-stride loops of many short blocks; persistent = 1: one resident wave of closest-hit and
 * occlusion kernels whose warps hand queue rays to lanes as lanes finish, each ray advancing at
 * most `budget` inner-node visits between hand-outs, a hand-out happening once `refill` lanes of
 * a warp are free (0: the defaults, 32 and 8). */
VGB_API vgb_status vgb_set_wavefront_tuning(vgb_context* ctx, uint32_t persistent, uint32_t budget, uint32_t refill);
/* Traversal steps (node visits) one ray may take before it gives up; 0 restores the default
 * of 2^22.  A ray past the limit stops, the call returns VGB_ERR_DEVICE_LIMIT with a message
 * and the context stays usable.  The limit exists so that no kernel can run unbounded on a
 * corrupt tree; a small value exercises that path on a healthy scene.  No counterpart in the
 * reference (Embree has no such limit). */
VGB_API vgb_status vgb_set_traversal_limit(vgb_context* ctx, uint32_t max_steps);

/* ========================= rasterizer =========================================
 * CPURasterizer::render (include/implementation/rendering/cpu_rasterizer.ipp:29-270) on the
 * device, for the uploaded scene (no BVH needed): every triangle is moved to the camera frame,
 * culled when a corner is behind the camera, projected, and its bounding box of integer pixel
 * coordinates (X, Y) -- pixel corners, as the reference samples -- tested with edge functions;
 * the closest fragment by interpolated distance wins, ties going to the earlier triangle, as the
 * reference's strict `<` over triangles in order gives.  The winner's passes: depth, alpha
 * (count / sample = 1/0 = +inf, the reference's value), albedo (vertex albedo x texture), the
 * face or smooth normal, triangle_id = triangle index + 1 (the reference counts from 1), and with
 * simulate_lighting the unshadowed direct radiance of the RNG-free light samples (total_radiance;
 * direct and indirect stay 0, as in the reference) and the received power.
 * Camera frame: p_cam = R^T (p - origin) in FP32 from the vgb_camera (the reference multiplies by
 * glm's FP32 inverse of the camera transform: equal up to rounding); projection
 * (x, y) = K (p_cam.x / p_cam.z, p_cam.y / p_cam.z, 1), mirrored in x when z_dir < 0 (Blender). */
typedef struct vgb_raster_options {
    float intrinsic[6];        /* rows of K with z_dir folded in: fx, kxy, px, kyx, fy, py (camera.ipp:1540-1556) */
    uint32_t simulate_lighting;
    uint32_t smooth_shading;
    uint32_t nbands;
    uint32_t pad;
} vgb_raster_options;

VGB_API vgb_status vgb_rasterize(vgb_context* ctx, const vgb_camera* cam, const vgb_light* lights, uint32_t nlights,
                                 const vgb_raster_options* opts, vgb_film* film);

/* ========================= DEM Quipu files (.qld) ==============================
 * Vira's on-disk DEM pyramid (include/implementation/quipu/dem_quipu.ipp,
 * include/implementation/quipu/quipu_io.ipp): the identifier "QUIPU", class id 2002, the
 * transformation (position, rotation, scale, FP64), the LoD count, an albedo flag, the
 * normal cone, a table of (GSD, byte offset) per LoD, then per LoD its DEMProjection,
 * heights stored as uint8 / uint16 fixed point or FP32 (LZ4 block or raw), and optional
 * albedo (constant, one uint8 plane or one uint8 plane per band).
 * Reading: the file is parsed and LZ4-decoded on the host (own decoder of the LZ4 block
 * format, bounds-checked); the quantised heights and albedo travel to the device, where the
 * fixed-point decode, DEMProjection::transformToWorld, the triangulation and the vertex
 * normals run.  Errors of the functions without a context are read with
 * vgb_quipu_last_error(). */
typedef struct vgb_quipu_dem vgb_quipu_dem;

#define VGB_QUIPU_MAX_LODS 64
#define VGB_QUIPU_NO_ALBEDO 0xFFFFFFFFu

typedef struct vgb_quipu_header {
    uint16_t class_id;          /* 2002 (VIRA_DEM_PYRAMID) */
    uint16_t num_lods;
    uint32_t has_albedos;
    double position[3];         /* transformation: translation */
    double rotation[9];         /* column-major 3x3 rotation */
    double scale[3];
    float normal[3];            /* normal cone of the coarsest LoD: mean direction ... */
    float cone_angle;           /* ... and half angle, radians */
} vgb_quipu_header;

typedef struct vgb_quipu_projection {   /* DEMProjection (include/vira/dems/dem_projection.hpp) */
    uint32_t width, height;             /* resolution */
    double pixel_scale[2];
    uint32_t tile_definitions[2];
    uint32_t tile_row, tile_col;
    double xoff, yoff, dx, dy;
    uint32_t is_ogr;                    /* map-projected (GDAL); vertices are not built for these */
    uint32_t pad;
    double row_col_rotation[2];
    double model_tie_point[2];
} vgb_quipu_projection;

typedef struct vgb_quipu_lod_info {
    double gsd;                 /* table-of-contents GSD (x) */
    uint64_t offset;            /* byte offset of the LoD block */
    uint32_t width, height;     /* resolution of the stored heights: the vertex grid */
    vgb_quipu_projection projection;   /* as stored (its resolution sets the grid's extent) */
    float height_min, height_max;
    uint32_t precision;         /* class id of the stored heights: 3 uint8, 4 uint16, 1 float */
    uint32_t compressed;        /* heights are an LZ4 block */
    uint32_t albedo_type;       /* 0 constant, 1 grey uint8 plane, 2 one uint8 plane per band;
                                   VGB_QUIPU_NO_ALBEDO when the file stores none */
    uint32_t albedo_channels;   /* planes of a type-2 albedo */
} vgb_quipu_lod_info;

typedef struct vgb_quipu_read_options {   /* DEMQuipuReaderOptions (quipu/dem_quipu.hpp) */
    uint32_t nbands;            /* TSpectral::size() of the reading program */
    uint32_t read_albedos;      /* 0: every vertex gets default_albedo */
    float default_albedo;       /* reference default 0.06 */
    float albedo_profile[VGB_MAX_BANDS];   /* multiplies a grey albedo plane per band (1.0 = none) */
} vgb_quipu_read_options;

/* DEMQuipu::DEMQuipu (dem_quipu.ipp:29-60) + an index of every LoD block. */
VGB_API vgb_status vgb_quipu_open(const char* path, vgb_quipu_dem** out);
VGB_API void vgb_quipu_close(vgb_quipu_dem* q);
VGB_API const char* vgb_quipu_last_error(void);
VGB_API vgb_status vgb_quipu_get_header(const vgb_quipu_dem* q, vgb_quipu_header* out);
VGB_API vgb_status vgb_quipu_get_lod(const vgb_quipu_dem* q, uint32_t lod, vgb_quipu_lod_info* out);
/* The LoD DEMQuipu::readBuffers picks for a required GSD (dem_quipu.ipp:136-152): the last of
 * the leading LoDs whose GSD is <= required, LoD 0 if none. */
VGB_API uint32_t vgb_quipu_select_lod(const vgb_quipu_dem* q, double required_gsd);
/* readDEMHeights + fixedToFloat (quipu_io.ipp:601-626, image_utils.ipp:509-527) on the host:
 * [H][W] floats, +inf where the stored code is 0. */
VGB_API vgb_status vgb_quipu_read_heights(vgb_quipu_dem* q, uint32_t lod, float* heights);
/* The LoD's albedo as the DEM holds it (readAlbedos_f / readAlbedos, quipu_io.ipp:643-702), on
 * the host: constant: nbands floats; grey: [H][W]; per band: [H][W][nbands] (nbands must equal
 * the stored channels).  VGB_ERR_NOT_READY when the file stores none. */
VGB_API vgb_status vgb_quipu_read_albedo(vgb_quipu_dem* q, uint32_t lod, uint32_t nbands, float* albedo);
/* DEMQuipu::readBuffers (dem_quipu.ipp:124-221) -> DEM::makeVertexBuffer / makeIndexBuffer
 * (dem.ipp:152-211) on the device: positions [H*W][3], per-vertex albedo [H*W][nbands] (NULL to
 * skip), vertex normals [H*W][3] (NULL to skip; Mesh::calculateNormals), indices [2(W-1)(H-1)][3]
 * of which *ntris are written.  Arrays device memory if on_device else host.  Non-OGR
 * projections only. */
VGB_API vgb_status vgb_quipu_read_mesh(vgb_context* ctx, vgb_quipu_dem* q, uint32_t lod,
                                       const vgb_quipu_read_options* opts, float* positions,
                                       float* vert_albedo, float* normals, uint32_t* indices,
                                       uint32_t* ntris, int on_device);

typedef struct vgb_quipu_lod_data {       /* one DEM of the pyramid to write */
    vgb_quipu_projection projection;      /* width/height give the heights' resolution */
    const float* heights;                 /* [H][W]; +inf / NaN = no data */
    uint32_t albedo_type;                 /* 0 constant, 1 grey plane, 2 plane per band */
    uint32_t nbands;                      /* bands of a constant or per-band albedo */
    const float* albedo;                  /* constant: nbands; grey: [H][W]; per band: [H][W][nbands] */
} vgb_quipu_lod_data;

/* DEMQuipu::write (dem_quipu.ipp:224-332): the pyramid finest first; heights quantised to
 * uint8 / uint16 when the height range over 255 / 65535 is below GSD / 50, else FP32; LZ4
 * block format when compress (own encoder).  The rotation is written as given (column-major). */
VGB_API vgb_status vgb_quipu_write(const char* path, const vgb_quipu_lod_data* lods, uint32_t nlods,
                                   const double position[3], const double rotation[9],
                                   const double scale[3], int write_albedos, int compress);

/* The LZ4 block format (no frame) as the reference uses it through LZ4_compress_default /
 * LZ4_decompress_safe (quipu_io.ipp:181-231): decompress returns the bytes written or -1 for
 * a malformed or overrunning block; compress returns the block size or 0 when dst_cap <
 * vgb_lz4_bound(n). */
VGB_API int64_t vgb_lz4_decompress(const void* src, uint64_t src_size, void* dst, uint64_t dst_cap);
VGB_API uint64_t vgb_lz4_bound(uint64_t n);
VGB_API uint64_t vgb_lz4_compress(const void* src, uint64_t n, void* dst, uint64_t dst_cap);

#ifdef __cplusplus
}
#endif

#endif /* VGB_H */
