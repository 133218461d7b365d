/*
 * librcv — GB300 (sm_103a) implementation of the recursive-control-variate
 * gradient step of "Recursive Control Variates for Inverse Rendering"
 * (Nicolet et al. 2023).  C ABI: plain pointers and sizes, no exceptions.
 *
 * Memory: every pointer documented as "device" is memory the caller allocated
 * on the current CUDA device (e.g. a torch tensor); the library never frees
 * caller memory and, apart from the entry points that say otherwise, never
 * allocates.  `stream` is a cudaStream_t (NULL = legacy default stream); all
 * calls are stream-ordered and return before the GPU work completes.
 *
 * Return codes: RCV_OK (0) or a negative RCV_ERR_* code; rcv_last_error()
 * returns a message for the calling thread's last failure.
 *
 * Each entry point names the reference interface it replaces (paths are
 * relative to the rgl-epfl/recursive_control_variates repository).
 */
#ifndef RCV_H
#define RCV_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define RCV_OK 0
#define RCV_ERR_INVALID (-1)     /* bad argument: maps to ValueError      */
#define RCV_ERR_CUDA (-2)        /* CUDA launch / runtime failure         */
#define RCV_ERR_UNSUPPORTED (-3) /* configuration not supported           */

/* Counters written by the tracers (optional, may be NULL): 64-bit device
 * array of RCV_COUNTER_COUNT entries, accumulated with atomics. */
#define RCV_COUNTER_PATHS 0       /* paths traced                               */
#define RCV_COUNTER_LOOKUPS 1     /* density lookups on the main path           */
#define RCV_COUNTER_NEE_LOOKUPS 2 /* density lookups inside ratio tracking      */
#define RCV_COUNTER_SCATTERS 3    /* real scattering events                     */
#define RCV_COUNTER_GRAD_EVENTS 4 /* adjoint: density gradient scatters         */
#define RCV_COUNTER_ALBEDO_EVENTS 5 /* adjoint: albedo gradient scatters        */
#define RCV_COUNTER_COUNT 8

/* Sub-sensors of a `batch` sensor (Mitsuba's batch sensor, used by every
 * grid scene of the reference, experiments.py:28-50). */
#define RCV_MAX_SENSORS 16

/* World-space pinhole frame: origin, forward direction, and the right / up
 * basis vectors already scaled by tan(fov_x/2) and tan(fov_x/2)*h/w of the
 * sensor's own film. */
typedef struct rcv_camera_frame {
  float origin[3];
  float forward[3];
  float right[3];
  float up[3];
} rcv_camera_frame;

/* Perspective pinhole sensor, or a batch of `count` of them rendering side
 * by side into one film.  Single sensor (count 0 or 1): pixel (x, y) with
 * film offset (u, v) maps to the direction
 * forward + (2(x+u)/width - 1) right + (1 - 2(y+v)/height) up.
 * Batch (count = n > 1, width a multiple of n): the film position
 * s = (x+u)/width selects sub-sensor k = min(floor(s n), n-1) and the
 * sub-sensor sees the position s n - floor(s n) of its own film; sub-sensor 0
 * is the frame of the fields below, sub-sensor k >= 1 is more[k-1]. */
typedef struct rcv_sensor {
  int32_t width;   /* film width (all sub-sensors)  */
  int32_t height;
  float origin[3];
  float forward[3];
  float right[3];
  float up[3];
  int32_t count;   /* sub-sensors: 0 or 1 = a single sensor, at most RCV_MAX_SENSORS */
  int32_t pad;
  rcv_camera_frame more[RCV_MAX_SENSORS - 1];
} rcv_sensor;

/* Two-state heterogeneous medium filling an axis-aligned box behind a null
 * boundary: the unit cube [0,1]^3 mapped by to_world = translate(box_min) *
 * scale(box_size) (the `to_world` of the reference's cube shape and grids,
 * experiments.py:57,64,79,285).  A box_size component of 0 means 1, so a
 * zero-initialised box is the unit cube.  Grids are x-fastest float32 arrays
 * of shape [Dz][Dy][Dx] (density) and [Dz][Dy][Dx][3] (albedo), sampled
 * trilinearly at voxel centres with clamp-to-edge.  sigma_t = scale *
 * density per unit world distance, sigma_s = albedo * sigma_t. */
typedef struct rcv_medium {
  int32_t dims[3]; /* Dx, Dy, Dz */
  float scale;
  const float* density_old; /* device, state theta_{i-1}                    */
  const float* density_new; /* device, state theta_i                        */
  const float* albedo_old;  /* device or NULL (then albedo_value is used)   */
  const float* albedo_new;  /* device or NULL                               */
  float albedo_value[3];
  /* 0: one global majorant (scale * max density).  f > 0: a majorant
   * supergrid of ceil(D/f) cells per axis traversed by DDA (the
   * `majorant_resolution_factor` of the reference's media,
   * plugins/twostatemedium.py:25-70); each cell holds scale * the largest
   * density trilinear interpolation can return inside it. */
  int32_t majorant_factor;
  void* workspace; /* device, rcv_medium_workspace_bytes(), 256-B aligned  */
  float box_min[3];  /* world position of the grid's (0,0,0) corner         */
  float box_size[3]; /* world extent along x, y, z (0 = 1)                  */
  /* Resolution of the albedo grids when it differs from the density's
   * (e.g. 264x136x136 density with 256x128x128 albedo, experiments.py:56,63);
   * all 0 = the density's.  Both grids span the same box. */
  int32_t albedo_dims[3];
  int32_t pad;
} rcv_medium;

/* Environment map (the reference's `envmap` emitter of its grid scenes,
 * experiments.py:81-85,195-199,315-319): a latitude-longitude RGB image of
 * linear radiance, times `scale`.  Row 0 is the +y pole, column u covers
 * azimuth 2 pi u: a world direction (x, y, z) has
 *   u = atan2(x, -z) / (2 pi) (wrapped into [0, 1)),  v = acos(y) / pi,
 * and the radiance is the bilinear interpolation of the texel centres
 * ((j + 1/2) / width, (i + 1/2) / height), wrapping in u and clamping in v.
 * Directions are importance-sampled from a piecewise-constant density over
 * the texels, proportional to luminance x sin(theta) of the texel's row
 * centre, whose solid-angle pdf is p(u, v) / (2 pi^2 sin(theta)).
 * rcv_envmap_prepare fills the workspace (texels with their sampling
 * weights, conditional and marginal CDFs) once after the texels change. */
typedef struct rcv_envmap {
  int32_t width, height;
  float scale;
  int32_t pad;
  const float* texels; /* device, [height][width][3] RGB                      */
  void* workspace;     /* device, rcv_envmap_workspace_bytes(), 256-B aligned  */
} rcv_envmap;

uint64_t rcv_envmap_workspace_bytes(int32_t width, int32_t height);
/* Builds the sampling tables of an environment map in its workspace (one
 * thread per row sums its texels in double, in order; one thread the rows).
 * No counterpart call in the reference: Mitsuba builds its envmap's
 * distribution when the plugin loads. */
int rcv_envmap_prepare(const rcv_envmap* envmap, void* stream);

typedef struct rcv_volpath_options {
  int32_t max_depth;     /* path length limit (real scattering events), -1 = none */
  int32_t rr_depth;      /* Russian roulette applies when depth > this            */
  int32_t hide_emitters; /* skip directly visible environment                     */
  int32_t batch;         /* paths a warp claims per queue fetch, 0 = 64           */
  int32_t blocks_per_sm; /* persistent blocks per SM, 0 = occupancy limit        */
  int32_t defer;         /* lanes that must wait before a path-start or
                            scattering branch runs, 1..32, 0 = 8                 */
  int32_t order;         /* pixel hand-out order, RCV_ORDER_*                     */
  int32_t count_events;  /* batched launches: accumulate the RCV_COUNTER_* totals
                            behind rcv_batch_counters (single-job calls count when
                            their `counters` argument is non-NULL)               */
  /* Environment emitter of the volume tracers and volpathsimple: a prepared
   * environment map, or NULL for the constant white environment (radiance
   * 1).  The batched engine takes the constant environment only. */
  const rcv_envmap* envmap;
  /* Adjoint of the single-job volume tracer (rcv_render_backward_volume and
   * the radiance / replay stages): RCV_ADJOINT_TAPE records every gradient
   * event of the radiance pass on a tape and scatters the gradient from it in
   * one flat pass; RCV_ADJOINT_REPLAY replays the paths' segments from
   * scattering checkpoints.  Both give the same gradient (up to the order of
   * float additions).  Under a majorant supergrid the tape keeps each
   * event's majorant beside it (at most 12 events per path); forward mode
   * and jobs (or batches) of 2^28 gradient paths or more always replay.  The
   * batched engine takes the same choice. */
  int32_t adjoint;
  /* Tape slots per path, 1..16 (0 = 16, the room the adjoint workspace
   * holds): paths whose events do not fit are replayed whole. */
  int32_t tape_events_per_path;
  /* The two-state pass and the adjoint's radiance pass of a step as two
   * launches (1; the batched engine runs them on two streams) instead of one
   * paired persistent launch (0, the default: the batched step, and
   * rcv_render_twostates_volume_and_adjoint_radiance).  The results are the
   * same either way. */
  int32_t separate_tracers;
} rcv_volpath_options;

#define RCV_ADJOINT_TAPE 0
#define RCV_ADJOINT_REPLAY 1

/* Pixel hand-out orders of the persistent tracers.  Results do not depend on
 * the order; it only changes how evenly the work drains at the end.
 * RCV_ORDER_COST hands out first the pixels whose paths took longest in the
 * previous call on the same workspace: each tracer call adds every path's
 * length (loop iterations) to a per-pixel cost array kept in the workspace,
 * and the next call sorts the pixels by it (then clears it).  A first call
 * finds whatever the workspace holds there; any content is valid and
 * changes only the schedule. */
#define RCV_ORDER_COST 0          /* most expensive pixels of the last call first */
#define RCV_ORDER_ROW_MAJOR 1
#define RCV_ORDER_LONGEST_FIRST 2 /* longest chord through the medium first     */

/* Tracer kinds for rcv_render_workspace_bytes. */
#define RCV_MODE_TWOSTATE 0
#define RCV_MODE_SINGLE 1
#define RCV_MODE_ADJOINT 2

/* ---------------------------------------------------------------- errors */
const char* rcv_last_error(void);
/* Number of kernels librcv has launched in this process (all streams). */
uint64_t rcv_kernel_launches(void);
/* Compute capability and SM count of the current device (no allocation). */
int rcv_device_info(int32_t* major, int32_t* minor, int32_t* sm_count);
/* sizeof() of a public struct by its type name ("rcv_sensor", ...), 0 for an
 * unknown name: lets foreign-function bindings check their layouts. */
uint64_t rcv_struct_size(const char* name);

/* -------------------------------------------------------------- sampling */
/* TEA hash (4 rounds); out[0] is what the reference uses as the default
 * gradient seed `mi.sample_tea_32(seed, 1)[0]`
 * (plugins/twostatepath.py:87-89). */
void rcv_sample_tea_32(uint32_t v0, uint32_t v1, uint32_t out[2]);

/* --------------------------------------------------------------- medium  */
/* Bytes of device workspace a medium needs (packed lookup cells, majorants,
 * gradient accumulators). */
uint64_t rcv_medium_workspace_bytes(const int32_t dims[3], int32_t has_albedo_grid, int32_t majorant_factor);
/* The same from a medium description (dims, albedo_dims, albedo_old != NULL,
 * majorant_factor); needed when the albedo grid has its own resolution. */
uint64_t rcv_medium_workspace_bytes_for(const rcv_medium* medium);

/* Packs the old/new grids into the lookup workspace and computes both
 * majorants (scale * max density).  Call after every state rotation.
 * Replaces the grid preparation Mitsuba performs in
 * TwoStateMedium.parameters_changed (plugins/twostatemedium.py:189-200) and
 * the majorant queries of sample_interaction_twostates
 * (plugins/twostatemedium.py:72-78). */
int rcv_medium_prepare(const rcv_medium* medium, void* stream);

/* ------------------------------------------------------------- tracers  */
/* Scratch a tracer call needs (work-queue counter, pixel order, per-pixel
 * cost and, for the primal tracers, one radiance slot per path; for the
 * adjoint 476 B per path: total radiance, 2 scatter checkpoints or event
 * records with their weights, 16 tape slots of 16 B each with a 4-B
 * extinction term, camera-segment weight, lost-path list): 256-B aligned device memory of this size, passed as
 * `workspace`.  The per-pixel cost persists from call to call
 * (RCV_ORDER_COST); pass the same workspace to the calls of one image size.
 * mode = RCV_MODE_*. */
uint64_t rcv_render_workspace_bytes(int32_t width, int32_t height, int32_t spp, int32_t mode);

/* Two-state primal: renders the previous (img_old = H) and current
 * (img_new = F) parameters with shared random numbers.  Images are
 * [height][width][3] float32 device arrays.
 * Replaces TwoStatePRBVolpathIntegrator.render_twostates /
 * sample_twostates / sample_emitter_twostates
 * (plugins/twostatevolpath.py:91-138, 141-385, 387-479). */
int rcv_render_twostates_volume(const rcv_medium* medium, const rcv_sensor* sensor,
                                const rcv_volpath_options* opts, uint32_t seed, int32_t spp,
                                float* img_old, float* img_new, void* workspace,
                                uint64_t* counters, void* stream);

/* Single-state primal on the current (new) parameters; the render that
 * `integrator.render(...)` of a two-state integrator performs (it delegates
 * every medium query to `new`, plugins/twostatemedium.py:125-151) and that
 * MetaIntegrator uses for force_baseline (plugins/metaintegrator.py:124-128). */
int rcv_render_volume(const rcv_medium* medium, const rcv_sensor* sensor,
                      const rcv_volpath_options* opts, uint32_t seed, int32_t spp, float* img,
                      void* workspace, uint64_t* counters, void* stream);

/* rcv_render_volume without caller scratch.  No counterpart in the reference:
 * it exists for callers that cannot allocate device memory — for example code
 * that runs where cudaMalloc is unavailable or forbidden, or a host that owns
 * a fixed memory pool and gives this library only its inputs and outputs.
 * Its scratch (work-queue counter, pixel order, per-path radiance) is a
 * file-scope static __device__ array of 16 MiB that every GPU loading the
 * library holds until exit.  A call needs 16 B per path and 8 B per pixel
 * (pixel order and pixel cost) plus under 2 KB of counters, buckets and
 * alignment; exactly, rcv_render_workspace_bytes(width, height, spp,
 * RCV_MODE_SINGLE) must not exceed 16 MiB.  Larger requests return
 * RCV_ERR_INVALID with the needed size.  It calls no allocator.  The first
 * call on each device looks up the array's device address
 * (cudaGetSymbolAddress) and keeps it; make that first call before any
 * stream capture.  The kept address belongs to the device's current primary
 * context: after cudaDeviceReset on a device, this entry point must not be
 * called again on that device in the same process.
 * All calls on one device share that device's copy of the array and find
 * the previous call's contents in it (the call resets what must start at
 * zero): calls that can overlap on the GPU, e.g. issued on two streams,
 * race and must be serialised by the caller.  The medium and its workspace
 * are inputs, as for rcv_render_volume. */
int rcv_render_volume_noalloc(const rcv_medium* medium, const rcv_sensor* sensor,
                              const rcv_volpath_options* opts, uint32_t seed, int32_t spp,
                              float* img, uint64_t* counters, void* stream);

/* Path-replay adjoint on the current parameters: traces `spp` paths per
 * pixel from `seed` to obtain each path's radiance, then back-propagates
 * grad_img (dLoss/dimage, [height][width][3]) into the density grid (and the
 * albedo grid when the medium has one) at every event of the paths: from the
 * event tape the radiance pass recorded (RCV_ADJOINT_TAPE, the default), or
 * by tracing the paths' segments again from scatter checkpoints
 * (RCV_ADJOINT_REPLAY).  Gradients are
 * ADDED to grad_density ([Dz][Dy][Dx]) and grad_albedo ([Dz][Dy][Dx][3] or
 * NULL).
 * Replaces CVIntegrator.render_backward / MetaIntegrator.render_backward
 * (plugins/cv_integrator.py:87-94, plugins/metaintegrator.py:140-147), i.e.
 * the path-replay adjoint of the wrapped two-state integrator. */
int rcv_render_backward_volume(const rcv_medium* medium, const rcv_sensor* sensor,
                               const rcv_volpath_options* opts, uint32_t seed, int32_t spp,
                               const float* grad_img, float* grad_density, float* grad_albedo,
                               void* workspace, uint64_t* counters, void* stream);

/* Forward-mode derivative of the single-state render on the current
 * parameters along a tangent of the density grid ([Dz][Dy][Dx], device, or
 * NULL) and / or of the albedo grid ([aDz][aDy][aDx][3], device, or NULL):
 * dimg ([height][width][3], overwritten) = d image / d epsilon at
 * theta + epsilon * tangent, estimated by path replay with `spp` paths per
 * pixel from `seed` (the same radiance pass as rcv_render_backward_volume,
 * then the replay tasks gather the tangent where the adjoint scatters).
 * The medium's gradient accumulators are overwritten.  Replaces
 * CVIntegrator.render_forward / MetaIntegrator.render_forward
 * (plugins/cv_integrator.py:79-85, plugins/metaintegrator.py:132-138), i.e.
 * the forward mode of the path-replay integrator. */
int rcv_render_forward_volume(const rcv_medium* medium, const rcv_sensor* sensor,
                              const rcv_volpath_options* opts, uint32_t seed, int32_t spp,
                              const float* tangent_density, const float* tangent_albedo, float* dimg,
                              void* workspace, uint64_t* counters, void* stream);

/* rcv_render_backward_volume in two calls.  The first pass of the adjoint
 * (each path's radiance and its event tape or scatter checkpoints) does not
 * depend on grad_img, so it can run as soon as the parameters are known — e.g.
 * on a second stream beside the primal render — and the second call, given
 * grad_img, only scatters the tape (or replays).  The replay call must get the same medium state,
 * sensor, options, seed, spp and workspace as the radiance call, and be
 * ordered after it; the pair gives the same gradients as
 * rcv_render_backward_volume. */
int rcv_render_adjoint_radiance(const rcv_medium* medium, const rcv_sensor* sensor,
                                const rcv_volpath_options* opts, uint32_t seed, int32_t spp,
                                void* workspace, uint64_t* counters, void* stream);
int rcv_render_backward_replay(const rcv_medium* medium, const rcv_sensor* sensor,
                               const rcv_volpath_options* opts, uint32_t seed, int32_t spp,
                               const float* grad_img, float* grad_density, float* grad_albedo,
                               void* workspace, uint64_t* counters, void* stream);

/* One optimisation step's two gradient-independent tracers in one call: the
 * two-state primal of (seed, spp) into img_old / img_new, exactly as
 * rcv_render_twostates_volume with `workspace`, and the adjoint's radiance
 * pass of (seed_grad, spp_grad), exactly as rcv_render_adjoint_radiance
 * with `adjoint_workspace` (a separate buffer of RCV_MODE_ADJOINT size).
 * rcv_render_backward_replay with (seed_grad, spp_grad, adjoint_workspace)
 * then completes the gradient.  Both tracers run in one persistent launch,
 * so that the longest paths of both start together instead of the second
 * launch's starting only as the first one's blocks retire; with event
 * counting (counters non-NULL), the replay adjoint or separate_tracers the
 * two run as separate launches.  Images and gradients equal those of the separate
 * calls.  Replaces the primal of the reference's cv_ps step
 * (TwoStatePRBVolpathIntegrator.render_twostates,
 * plugins/twostatevolpath.py:91-138) together with the primal phase that the
 * path-replay adjoint runs before its backward phase (render_backward of
 * the prb_volpath integrator it derives from). */
int rcv_render_twostates_volume_and_adjoint_radiance(const rcv_medium* medium, const rcv_sensor* sensor,
                                                     const rcv_volpath_options* opts, uint32_t seed,
                                                     int32_t spp, float* img_old, float* img_new,
                                                     void* workspace, uint32_t seed_grad, int32_t spp_grad,
                                                     void* adjoint_workspace, uint64_t* counters, void* stream);

/* ------------------------------------------------ volpathsimple integrator */
/* Switches of VolpathSimpleIntegrator (plugins/volpathsimple.py:20-51):
 * use_nee, use_drt, use_drt_subsampling, use_drt_mis (each 0 or 1; the
 * reference's defaults are all 1).  NULL selects the defaults. */
typedef struct rcv_volpathsimple_flags {
  int32_t use_nee, use_drt, use_drt_subsampling, use_drt_mis;
} rcv_volpathsimple_flags;

/* Scratch of rcv_render_volpathsimple: 16 bytes per path. */
uint64_t rcv_volpathsimple_workspace_bytes(int32_t width, int32_t height, int32_t spp);

/* Primal of the simplified volumetric path tracer on the current (new)
 * parameters: delta tracking to real interactions, NEE towards the
 * environment, MIS at the environment.  Replaces
 * VolpathSimpleIntegrator.sample (plugins/volpathsimple.py:53-327). */
int rcv_render_volpathsimple(const rcv_medium* medium, const rcv_sensor* sensor,
                             const rcv_volpath_options* opts, const rcv_volpathsimple_flags* flags,
                             uint32_t seed, int32_t spp, float* img, void* workspace, void* stream);

/* Adjoint of the simplified tracer: path replay with the scattering,
 * transmittance and NEE terms and differential ratio tracking.  Gradients
 * as rcv_render_backward_volume.  Replaces the render_backward of the
 * `adjoint_integrator` built from {"type": "volpathsimple"}
 * (plugins/volpathsimple.py:53-327, 508-778; experiments.py:131,245,364). */
int rcv_render_backward_volpathsimple(const rcv_medium* medium, const rcv_sensor* sensor,
                                      const rcv_volpath_options* opts,
                                      const rcv_volpathsimple_flags* flags, uint32_t seed,
                                      int32_t spp, const float* grad_img, float* grad_density,
                                      float* grad_albedo, void* stream);

/* ------------------------------------------------------- surface scenes */
#define RCV_MAX_SPHERES 8

typedef struct rcv_sphere {
  float center[3];
  float radius;
  float albedo[3]; /* diffuse reflectance (equal in both states) */
} rcv_sphere;

/* Ground rectangle y = 0, |x|,|z| <= plane_half, with a two-state diffuse
 * RGB texture (u along x, v along z, bilinear, repeat wrap), diffuse spheres
 * and one rectangular area light at y = light_center[1] facing -y. */
typedef struct rcv_surface_scene {
  float plane_half;
  int32_t tex_width;
  int32_t tex_height;
  const float* tex_old; /* device [tex_height][tex_width][3], state theta_{i-1} */
  const float* tex_new; /* device, state theta_i                              */
  int32_t num_spheres;  /* <= RCV_MAX_SPHERES */
  rcv_sphere spheres[RCV_MAX_SPHERES];
  float light_center[3];
  float light_half[2]; /* half extents along x and z */
  float light_radiance[3];
  void* workspace; /* device, rcv_surface_workspace_bytes(), 256-B aligned */
} rcv_surface_scene;

/* Workspace of a surface scene: texture state pairs and gradient. */
uint64_t rcv_surface_workspace_bytes(int32_t tex_width, int32_t tex_height);

/* Packs the old / new textures after a state rotation
 * (TwoStateBSDF.parameters_changed, plugins/twostatebsdf.py:46-56). */
int rcv_surface_prepare(const rcv_surface_scene* scene, void* stream);

/* Two-state surface primal (H = old, F = new), replacing
 * TwoStatePRBIntegrator.render_twostates / sample_twostates
 * (plugins/twostatepath.py:179-223, 225-364) with the two-state BSDF of
 * plugins/twostatebsdf.py:25-38.  Scratch: rcv_render_workspace_bytes(...,
 * RCV_MODE_TWOSTATE). */
int rcv_render_twostates_surface(const rcv_surface_scene* scene, const rcv_sensor* sensor,
                                 const rcv_volpath_options* opts, uint32_t seed, int32_t spp,
                                 float* img_old, float* img_new, void* workspace,
                                 uint64_t* counters, void* stream);

/* Single-state surface render of `new` (TwoStatePRBIntegrator.render). */
int rcv_render_surface(const rcv_surface_scene* scene, const rcv_sensor* sensor,
                       const rcv_volpath_options* opts, uint32_t seed, int32_t spp, float* img,
                       void* workspace, uint64_t* counters, void* stream);

/* Path-replay adjoint of the surface render on `new`: ADDS dLoss/dtexture to
 * grad_texture ([tex_height][tex_width][3]); replaces
 * CVIntegrator.render_backward with a twostateprb integrator
 * (plugins/cv_integrator.py:87-94, Mitsuba PRBIntegrator.render_backward).
 * opts->adjoint: RCV_ADJOINT_TAPE traces each path once, recording its
 * texture vertices (2 of the 16 tape slots per path each), and scatters them
 * once L is known; RCV_ADJOINT_REPLAY traces each path a second time.
 * Scratch: rcv_render_workspace_bytes(..., RCV_MODE_ADJOINT). */
int rcv_render_backward_surface(const rcv_surface_scene* scene, const rcv_sensor* sensor,
                                const rcv_volpath_options* opts, uint32_t seed, int32_t spp,
                                const float* grad_img, float* grad_texture, void* workspace,
                                uint64_t* counters, void* stream);

/* Forward-mode derivative of the surface render on `new` along a texture
 * tangent ([tex_height][tex_width][3], device): dimg ([height][width][3],
 * overwritten) by path replay, as rcv_render_forward_volume.  The scene's
 * texture gradient record is overwritten.  Replaces the render_forward of
 * the surface integrator behind cv / meta (plugins/cv_integrator.py:79-85). */
int rcv_render_forward_surface(const rcv_surface_scene* scene, const rcv_sensor* sensor,
                               const rcv_volpath_options* opts, uint32_t seed, int32_t spp,
                               const float* tangent_texture, float* dimg, void* workspace,
                               uint64_t* counters, void* stream);

/* ------------------------------------------------- control variate state */
/* Per-element state of the recursive control variate; every array holds
 * `n` float32 device values (n = height*width*3), zero-initialised. */
typedef struct rcv_cv_state {
  float* img;    /* G_{i-1} -> G_i                                        */
  float* w_s;    /* control weight alpha                                  */
  float* v_n;    /* variance of the previous estimate                     */
  float* mean_x; /* EMA-Welford statistics of H (x) and F (y)             */
  float* mean_y;
  float* var_x;
  float* var_y;
  float* cov;
} rcv_cv_state;

/* One control-variate step: optional statistics update (pre_update), weight
 * update when it > warmup, the blend img = w_s (img - H) + F, then the
 * statistics update when it > 0.  *welford_count (host memory) is the
 * estimator's sample count n and is incremented by every update.
 * Replaces CVIntegrator.render (plugins/cv_integrator.py:58-77), the cv_ps
 * branch of MetaIntegrator.render (plugins/metaintegrator.py:93-113) and
 * StatisticsEstimator.update / get (plugins/welford.py:59-78). */
int rcv_cv_step(const rcv_cv_state* state, int64_t n, const float* H, const float* F,
                int32_t it, int32_t warmup, int32_t* welford_count, float beta1, float beta2,
                int32_t pre_update, void* stream);

/* StatisticsEstimator.get (plugins/welford.py:77-78): bias-corrected
 * (var_x, var_y, cov) written to out_vx / out_vy / out_cov. */
int rcv_statistics_get(const rcv_cv_state* state, int64_t n, int32_t welford_count, float beta2,
                       float* out_vx, float* out_vy, float* out_cov, void* stream);

/* StatisticsEstimator.update (plugins/welford.py:59-75) on its own: updates
 * mean_x/mean_y/var_x/var_y/cov of `state` from x (= H) and y (= F) and
 * increments *welford_count; img / w_s / v_n are untouched. */
int rcv_statistics_update(const rcv_cv_state* state, int64_t n, const float* x, const float* y,
                          int32_t* welford_count, float beta1, float beta2, void* stream);

/* WelfordVarianceEstimator.update / get (plugins/welford.py:25-36). */
int rcv_welford_update(float* mean, float* var, int64_t n, const float* x, int32_t* count,
                       float beta1, float beta2, void* stream);
int rcv_welford_get(const float* var, int64_t n, int32_t count, float beta2, float* out,
                    void* stream);

/* --------------------------------------------------------- step harness */
#define RCV_LOSS_L2 0
#define RCV_LOSS_L1 1
/* Workspace bytes rcv_loss needs for a deterministic two-stage reduction. */
uint64_t rcv_loss_workspace_bytes(int64_t n);
/* loss = mean((img-ref)^2) or mean(|img-ref|) into *loss (device float);
 * grad (device, n, or NULL) = dloss/dimg.  Replaces utils.l2_loss / l1_loss
 * (utils.py:21-25) and their derivative d_l (utils.py:90-96). */
int rcv_loss(int32_t kind, const float* img, const float* ref, int64_t n, float* loss, float* grad,
             void* workspace, void* stream);

/* Adam step with the bias correction folded into the step size, followed by
 * clamping to [lo, hi] and (optionally) zeroing grad.  `t` is the 1-based
 * step count.  Replaces mi.ad.Adam.step (optimize.py:90,127) and
 * utils.clamp (utils.py:172-175). */
int rcv_adam_step(float* param, float* grad, float* m, float* v, int64_t n, int32_t t, float lr,
                  float beta1, float beta2, float eps, float lo, float hi, int32_t zero_grad,
                  void* stream);

/* x = min(max(x, lo), hi) elementwise (utils.clamp, utils.py:172-175). */
int rcv_clamp(float* x, int64_t n, float lo, float hi, void* stream);

/* ---------------------------------------------------- bias-correction tables
 * The batched engine derives every per-step scalar on the device from step
 * counters, so the powers beta^k that rcv_cv_step and rcv_adam_step compute on
 * the host come from tables filled here with the same host arithmetic.
 *
 * CV table of beta: d[k] = 1 - float32(beta^k), k = 0..len-1, where len-1 is
 * the first k with d[k] == 1.0f (every later power gives 1.0f as well).
 * Adam table of (beta1, beta2): two doubles per t = 0..len-1,
 * (sqrt(1 - beta2^t), 1 - beta1^t), ending at the first t where both are 1.0.
 * The _len functions return the entry count, or RCV_ERR_UNSUPPORTED when beta
 * is so close to 1 that the table would exceed 2^22 entries, or
 * RCV_ERR_INVALID for beta outside [0, 1).  _fill writes `len` entries into
 * host memory. */
int64_t rcv_cv_table_len(float beta);
int rcv_cv_table_fill(float beta, float* out, int64_t len);
int64_t rcv_adam_table_len(float beta1, float beta2);
int rcv_adam_table_fill(float beta1, float beta2, double* out, int64_t len);

/* ------------------------------------------------------ batched cv_ps steps
 * Many independent optimisation jobs (each a cv_ps loop of optimize.py:
 * params.update, mi.render with the cv integrator around twostateprbvolpath,
 * l2/l1 loss, dr.backward, Adam + clamp) advanced together: one step of the
 * batch is one step of every job, in six kernel launches whatever the number
 * of jobs (nine with the per-step pixel sort of RCV_ORDER_COST): a prologue
 * that derives each job's seeds and CV / Adam scalars from
 * its device counters, the medium packing of all jobs, ONE persistent
 * two-state tracer launch over the paths of all jobs, one fused
 * reduce + control-variate + loss kernel, ONE persistent adjoint launch and
 * one fused gradient fold + Adam + clamp kernel.  No host value changes from
 * step to step, so the step can be captured once into a CUDA graph and
 * replayed.  Per job and step the results equal the single-job calls
 * (rcv_render_twostates_volume, rcv_cv_step, rcv_loss,
 * rcv_render_backward_volume, rcv_adam_step) with seed = seed_base + it and
 * seed_grad = sample_tea_32(seed, 1)[0] (plugins/twostatepath.py:84-92); the
 * images are identical, the gradients agree up to the order of float atomics.
 * Replaces the per-iteration loop body of optimize.py:105-131 for many jobs;
 * the reference has no batched form. */

/* One job.  All pointers are device memory owned by the caller. */
typedef struct rcv_batch_job {
  rcv_sensor sensor;
  int32_t dims[3];         /* density grid Dx, Dy, Dz                             */
  float scale;             /* sigma_t = scale * density                           */
  float albedo_value[3];   /* constant albedo when albedo[0] is NULL              */
  int32_t spp, spp_grad;   /* primal / adjoint samples per pixel                  */
  int32_t max_depth, rr_depth, hide_emitters;
  uint32_t seed_base;      /* step `it` renders with seed = seed_base + it        */
  int32_t warmup;          /* cv plugin: weights update when it > warmup          */
  int32_t pre_update;      /* meta cv_ps: statistics update before the weight     */
  float cv_beta1, cv_beta2;
  const float* cv_table1;  /* rcv_cv_table_fill(cv_beta1) copied to the device    */
  const float* cv_table2;  /* rcv_cv_table_fill(cv_beta2)                         */
  int32_t cv_table1_len, cv_table2_len;
  int32_t loss;            /* RCV_LOSS_L2 / RCV_LOSS_L1 against `target`          */
  float lr, adam_beta1, adam_beta2, adam_eps;
  float density_lo, density_hi, albedo_lo, albedo_hi; /* clamp ranges             */
  const double* adam_table; /* rcv_adam_table_fill(adam_beta1, adam_beta2)        */
  int32_t adam_table_len;
  int32_t majorant_factor;  /* as rcv_medium.majorant_factor                      */
  float box_min[3];         /* as rcv_medium.box_min / box_size                   */
  float box_size[3];
  /* Parameters, double-buffered: before step `it`, density[it & 1] holds
   * theta_it (the `new` state) and density[(it & 1) ^ 1] holds theta_{it-1}
   * (`old`); the step writes theta_{it+1} into the latter.  Both buffers hold
   * the initial grid before the first step (old = new = initial state, as
   * the reference's double initialize_parameters, utils.py:62-66). */
  float* density[2];       /* D^3 each                                            */
  float* albedo[2];        /* D^3 * 3 each, or both NULL                          */
  float* density_m;        /* Adam moments, zero before the first step            */
  float* density_v;
  float* albedo_m;         /* NULL: the albedo is not optimised (then albedo[0]   */
  float* albedo_v;         /* and albedo[1] hold the same grid, may be one buffer) */
  const float* target;     /* (H, W, 3) reference image                           */
  rcv_cv_state cv;         /* (H, W, 3) each, zero before the first step          */
  float* img_old;          /* optional H output (NULL = not written)              */
  float* img_new;          /* optional F output                                   */
  void* workspace;         /* rcv_batch_job_workspace_bytes(), 256-B aligned      */
} rcv_batch_job;

/* Status at the start of a job workspace (device memory; read it with a
 * device-to-host copy). */
typedef struct rcv_batch_job_status {
  int32_t it;             /* steps taken; density[it & 1] holds theta_it          */
  int32_t welford_count;  /* the CV statistics' sample count n                    */
  int32_t adam_t;         /* Adam steps taken                                     */
  int32_t pad;
  double loss_sum;        /* sum of the last step's per-element losses            */
  float loss;             /* mean loss of the last step                           */
  float pad1;
} rcv_batch_job_status;

uint64_t rcv_batch_job_workspace_bytes(const rcv_batch_job* job);
/* Validates the job, zeroes its status, computes its longest-chord-first
 * pixel order (camera geometry only) and seeds its per-pixel cost with it. */
int rcv_batch_job_init(const rcv_batch_job* job, void* stream);

typedef struct rcv_batch rcv_batch; /* opaque host handle of a batch plan */

/* Shared device scratch of a batch: job tables, the per-path radiance of the
 * two-state launch (32 bytes per primal path of all jobs) and the adjoint's
 * per-path scratch (476 bytes per gradient path, as for
 * rcv_render_workspace_bytes).  opts->adjoint selects the tape or the replay
 * tasks for the whole batch. */
uint64_t rcv_batch_workspace_bytes(const rcv_batch_job* jobs, int32_t n);
/* Plans a batch of n initialised jobs with launch options `opts` (batch,
 * blocks_per_sm, defer, order; max_depth / rr_depth / hide_emitters come from
 * each job; NULL = defaults with RCV_ORDER_COST).  The per-pixel costs and
 * pixel orders live in the job workspaces.  Copies the job tables into `workspace` on `stream`; the host
 * array `jobs` may be freed on return.  *out is released by rcv_batch_destroy.
 * This is the one entry point group that allocates: host memory for the plan
 * and, when graphs are used, the CUDA graph. */
int rcv_batch_create(const rcv_batch_job* jobs, int32_t n, const rcv_volpath_options* opts,
                     void* workspace, uint64_t workspace_bytes, rcv_batch** out, void* stream);
/* One step of every job.  use_graph != 0: the first call captures the six
 * launches into a CUDA graph (on an internal stream, nothing runs), every
 * call launches the graph on `stream`. */
int rcv_batch_step(rcv_batch* batch, int32_t use_graph, void* stream);
/* Device pointer to 2 * RCV_COUNTER_COUNT uint64 tracer counters accumulated
 * over all steps: the two-state launch, then the adjoint launch. */
uint64_t* rcv_batch_counters(rcv_batch* batch);
/* Kernel launches one step of this batch issues (graph replays count the
 * same): six, plus three that sort each job's pixels with RCV_ORDER_COST. */
int32_t rcv_batch_kernels_per_step(const rcv_batch* batch);
int rcv_batch_destroy(rcv_batch* batch);

#ifdef __cplusplus
}
#endif
#endif /* RCV_H */
