/*
 * optika_gb300 C-ABI: the drop-in boundary of the GB300 sequential raytracer.
 *
 * Every entry point takes plain pointers and sizes (device pointers for ray
 * and image buffers, a host pointer for the packed system descriptor) and a
 * cudaStream_t passed as `void*`.  Nothing here allocates device memory on
 * the hot path; every buffer is owned by the caller.
 *
 * The reference (optika, pure Python) has no FFI.  Each function below
 * replaces a Python call chain of the reference, cited beside it
 * (file:line within the optika project).  Units are fixed: lengths in mm,
 * vacuum wavelengths in nm, angles in radians, attenuation in 1/mm.
 */
#ifndef OPTIKA_GB300_H
#define OPTIKA_GB300_H

#include <stdint.h>
#include <stddef.h>

#ifdef __cplusplus
extern "C" {
#endif

#define OTX_ABI_VERSION 3

#define OTX_MAX_SURFACES 16
#define OTX_MAX_POLY_TERMS 8
#define OTX_MAX_VERTICES 64
#define OTX_MAX_LAYERS 64
#define OTX_MAX_STACKS 4

/* ---- status codes ---------------------------------------------------- */
typedef int32_t otx_status;
#define OTX_OK 0
#define OTX_ERR_INVALID 1     /* bad descriptor or argument              */
#define OTX_ERR_UNSUPPORTED 2 /* a type tag this build does not know      */
#define OTX_ERR_CUDA 3        /* a CUDA runtime call failed              */
#define OTX_ERR_SIZE 4        /* a size exceeds a documented maximum      */
#define OTX_ERR_TIMEOUT 5     /* a bounded device wait gave up            */

/* ---- type tags ------------------------------------------------------- */
#define OTX_SAG_FLAT 0     /* optika/sags/_flat.py:13              NoSag        */
#define OTX_SAG_SPHERE 1   /* optika/sags/_spherical.py:40         SphericalSag */
#define OTX_SAG_CONIC 2    /* optika/sags/_conic.py:16             ConicSag     */
#define OTX_SAG_PARABOLA 3 /* optika/sags/_parabolic.py:14         ParabolicSag */
#define OTX_SAG_TOROID 4   /* optika/sags/_toroidal.py:14          ToroidalSag  */
#define OTX_SAG_CYLINDER 5 /* optika/sags/_cylindrical.py:14       CylindricalSag */

#define OTX_MAT_VACUUM 0            /* optika/materials/_materials.py:82  */
#define OTX_MAT_MIRROR 1            /* optika/materials/_materials.py:161 */
#define OTX_MAT_GLASS 2             /* optika/materials/_materials.py:309 */
#define OTX_MAT_MULTILAYER_MIRROR 3 /* optika/materials/_multilayers.py:908 */
#define OTX_MAT_MULTILAYER_FILM 4   /* optika/materials/_multilayers.py:839 */
#define OTX_MAT_MEASURED_MIRROR 5   /* optika/materials/_materials.py:177 */

#define OTX_APER_NONE 0
#define OTX_APER_CIRCULAR 1    /* optika/apertures/_apertures.py:292 */
#define OTX_APER_RECTANGULAR 2 /* optika/apertures/_apertures.py:941 */
#define OTX_APER_ELLIPTICAL 3  /* optika/apertures/_apertures.py:640 */
#define OTX_APER_SECTOR 4      /* optika/apertures/_apertures.py:438 */
#define OTX_APER_POLYGON 5     /* optika/apertures/_apertures.py:739 */

#define OTX_APER_FLAG_INVERTED 1
#define OTX_APER_FLAG_ACTIVE 2
#define OTX_APER_FLAG_DIRECTION 4 /* dimensionless aperture: tests direction */
#define OTX_APER_FLAG_TRANSFORM 8 /* apply `aper_to_local` before the test   */

#define OTX_RULE_NONE 0
#define OTX_RULE_CONSTANT 1    /* optika/rulings/_spacing.py:45  */
#define OTX_RULE_POLY1D 2      /* optika/rulings/_spacing.py:78  */
#define OTX_RULE_HOLOGRAPHIC 3 /* optika/rulings/_spacing.py:132 */

/* Groove-efficiency models of the rulings (optika/rulings/_rulings.py).  */
#define OTX_RULE_EFF_IDEAL 0       /* Rulings: rule_efficiency, :225       */
#define OTX_RULE_EFF_MEASURED 1    /* MeasuredRulings (table), :255        */
#define OTX_RULE_EFF_SINUSOIDAL 2  /* SinusoidalRulings, :317              */
#define OTX_RULE_EFF_SQUARE 3      /* SquareRulings, :461                  */
#define OTX_RULE_EFF_SAWTOOTH 4    /* SawtoothRulings, :618                */
#define OTX_RULE_EFF_TRIANGULAR 5  /* TriangularRulings, :762              */
#define OTX_RULE_EFF_RECTANGULAR 6 /* RectangularRulings, :915             */

#define OTX_SYS_FLAG_FINAL_IDENTITY 1 /* final_to_output is the identity */

#define OTX_INPUT_RAYS 0         /* full ray state, optika/surfaces.py:123     */
#define OTX_INPUT_GRID_INFINITY 1 /* object at infinity, _sequential.py:802-806 */
#define OTX_INPUT_GRID_FINITE 2   /* finite object,      _sequential.py:807-809 */

/* ---- descriptors ----------------------------------------------------- */

/* Rigid affine map x' = (m + m_lo) x + (t_hi + t_lo).  Composed on the
 * host in float64 and split into float-float parts so that the large
 * offsets between surfaces are added, and directions rotated, without
 * FP32 rounding. */
#define OTX_AFFINE_ROT_IDENTITY 1 /* m is exactly the identity           */
#define OTX_AFFINE_ROT_Y 2        /* m is a rotation about y: its middle   */
                                  /* row and column are exactly (0, 1, 0) */
#define OTX_AFFINE_IDENTITY 4     /* the whole map is exactly the identity */
typedef struct otx_affine {
  float m[9];    /* row-major 3x3 rotation, high parts */
  float m_lo[9]; /* low parts                          */
  float t_hi[3];
  float t_lo[3];
  int32_t flags;
  int32_t pad_;
} otx_affine; /* 104 bytes */

/* Complex refractive index source of one layer or substrate.  A negative
 * `table` means the constant n_re + i n_im; otherwise the index of a
 * (wavelength, n, k) table in otx_system.tables, linearly interpolated and
 * clamped at the ends (optika/chemicals/_chemicals.py:138-142). */
/* Interface profiles between layers (Stearns 1989), on the left side of a
 * layer: the layer's reflection amplitude r_ij is multiplied by the Fourier
 * transform of the profile's derivative (optika/materials/profiles.py). */
#define OTX_PROFILE_NONE 0
#define OTX_PROFILE_ERF 1         /* ErfInterfaceProfile, :130         */
#define OTX_PROFILE_EXPONENTIAL 2 /* ExponentialInterfaceProfile, :226 */
#define OTX_PROFILE_LINEAR 3      /* LinearInterfaceProfile, :328      */
#define OTX_PROFILE_SINUSOIDAL 4  /* SinusoidalInterfaceProfile, :434  */

typedef struct otx_layer {
  float n_re;
  float n_im;
  float thickness; /* nm */
  int32_t table;
  int32_t interface_type; /* OTX_PROFILE_* of the interface on its left */
  float interface_width;  /* nm */
} otx_layer;

/* A multilayer stack: `pre` layers, then `per` layers repeated
 * `num_periods` times, then `post` layers, on the substrate layer
 * (optika/materials/_layers.py:473-499, 611-645). */
typedef struct otx_stack {
  int32_t pre_begin, pre_count;
  int32_t per_begin, per_count, num_periods;
  int32_t post_begin, post_count;
  int32_t substrate; /* layer index, or -1 for vacuum */
} otx_stack;

/* One periodic bilayer mirror: [A, B] x num_periods on a substrate, with
 * constant complex indices (optika/materials/_layers.py:571-645 with two
 * layers of constant index). */
typedef struct otx_periodic_stack {
  float n_a_re, n_a_im, n_b_re, n_b_im, n_sub_re, n_sub_im;
  float thickness_a, thickness_b; /* nm */
  int32_t num_periods;
  int32_t pad_;
} otx_periodic_stack;

typedef struct otx_table {
  int32_t offset; /* into otx_system.table_data: [wl(n), n(n), k(n)] */
  int32_t count;
} otx_table;

typedef struct otx_surface {
  otx_affine to_local;  /* previous frame -> this surface's frame        */
  otx_affine to_output; /* this surface's frame -> output frame          */
  otx_affine aper_to_local; /* surface frame -> aperture frame             */
  otx_affine rule_xform;    /* polynomial-spacing argument transformation */

  /* sag */
  int32_t sag_type;
  float sag_radius;    /* R (sphere), 2f (parabola)                          */
  float sag_curvature; /* c = 1/R (sphere, conic, cylinder, toroid minor radius) */
  float sag_conic;     /* k                                                  */
  float sag_radius_of_rotation; /* toroid major radius                       */
  float sag_focal_length;       /* parabola                                  */

  /* material */
  int32_t mat_type;
  int32_t mat_is_mirror;
  int32_t mat_stack; /* index into otx_system.stacks (multilayer types)      */
  int32_t mat_table; /* measured mirror: index into tables,
                        columns [wavelength nm, reflectivity, unused]        */
  float sellmeier_b[3];
  float sellmeier_c[3]; /* nm^2 */

  /* aperture */
  int32_t aper_type;
  int32_t aper_flags;
  float aper_p[4]; /* circular: r | rect: hx,hy | ellipse: rx,ry |
                      sector: r, start, stop */
  int32_t aper_vertex_begin, aper_vertex_count;

  /* rulings */
  int32_t rule_type;
  int32_t rule_num_terms;
  float rule_order;      /* diffraction order m                         */
  float rule_efficiency; /* 1 for ideal rulings                          */
  float rule_normal[3];  /* unit normal of the ruling planes             */
  float rule_coef[OTX_MAX_POLY_TERMS]; /* d(x) = sum coef[k] x^k (mm)    */
  float holo_x1[3], holo_x2[3];
  float holo_wavelength; /* mm */
  float holo_d1, holo_d2; /* +1 diverging, -1 converging */
  int32_t rule_eff_type;  /* OTX_RULE_EFF_*                              */
  int32_t rule_table;     /* measured efficiency: index into tables,
                             columns [wavelength nm, efficiency, unused] */
  float rule_depth;       /* groove depth / model amplitude (nm)         */
  float rule_duty;        /* rectangular: a = 2 pi duty ratio (rad)      */

  int32_t is_sensor; /* bin rays leaving this surface (must be the last) */
  int32_t pad_;
} otx_surface;

typedef struct otx_sensor {
  int32_t num_x, num_y, num_w; /* pixels along x, y; wavelength bins    */
  int32_t pad_;
  float lo_x, lo_y;  /* lower edges (mm)                                */
  float width_x, width_y; /* pixel pitch (mm)                           */
  float w_lo, w_hi;  /* wavelength edges (nm), num_w uniform bins       */
  float inv_width_x, inv_width_y; /* 1 / pitch (derived by the library) */
  float inv_width_w;              /* num_w / (w_hi - w_lo) (derived)    */
  int32_t pad2_;
} otx_sensor;

typedef struct otx_system {
  int32_t abi_version;
  int32_t num_surfaces;
  int32_t input_mode; /* OTX_INPUT_*                                      */
  int32_t newton_iterations; /* max toroid Newton steps (0 = default 12) */
  int32_t flags;              /* OTX_SYS_FLAG_*                          */
  int32_t pad_;
  otx_affine final_to_output; /* last surface frame -> final output frame */
  otx_sensor sensor;
  otx_surface surfaces[OTX_MAX_SURFACES];
  float vertices[2 * OTX_MAX_VERTICES]; /* polygon apertures (x,y pairs) */
  otx_layer layers[OTX_MAX_LAYERS];
  otx_stack stacks[OTX_MAX_STACKS];
  otx_table tables[OTX_MAX_STACKS * 4];
  uint64_t table_data; /* device pointer to float table storage          */
} otx_system;

/* Structure-of-arrays ray buffers (device pointers).  Any pointer may be
 * null: an input then takes the reference's default (intensity 1,
 * attenuation 0, index 1, unvignetted true), an output is not written.
 * `stride_*` of 0 broadcasts element 0 (a scalar input). */
typedef struct otx_rays {
  uint64_t px, py, pz;      /* float* */
  uint64_t dx, dy, dz;      /* float* */
  uint64_t wavelength;      /* float* nm */
  uint64_t intensity;       /* float*    */
  uint64_t attenuation;     /* float* 1/mm */
  uint64_t index_refraction;/* float*    */
  uint64_t unvignetted;     /* uint8_t*  */
  uint64_t opl;             /* double*   optical path length (mm)       */
  int64_t count;
  int64_t surface_stride;   /* elements between surfaces when accumulating */
} otx_rays;

/* Grid inputs of SequentialSystem.raytrace (float* device arrays, each
 * with its own element stride, 0 = broadcast). */
typedef struct otx_grid {
  uint64_t wavelength, field_x, field_y, pupil_x, pupil_y, intensity;
  int64_t stride_wavelength, stride_field, stride_pupil, stride_intensity;
  int64_t count;
} otx_grid;

/* Sensor images, each [num_w][num_x][num_y] or 0 (not produced):
 * counts: uint32 ray counts; flux: float sum of intensity (the reference's
 * image, optika/sensors/_sensors.py:155); cos_moment: float sum of intensity
 * times the cosine of incidence on the sensor, -direction . normal (the
 * refracted cosine of an ideal sensor material, :156-169 and
 * optika/sensors/materials/_materials.py:1603-1616). */
typedef struct otx_image {
  uint64_t counts;
  uint64_t flux;
  uint64_t cos_moment;
} otx_image;

/* Batched trace of many configurations of one system shape.  Each config
 * replaces num_overrides surfaces of the base system (at override_index)
 * with its own descriptors; its rays are generated on the device by
 * Philox4x32-10 keyed by (seed, config) and counted by ray index:
 * wavelength U[wl_lo, wl_hi), field angles U[-half, half) in x and y,
 * pupil U[-pupil_half, pupil_half)^2.  Work items are tiles of up to
 * tile_size rays of one config, listed in `tiles`, taken by persistent CTAs
 * from the device counter `counter` (a uint32 the entry point clears). */
#define OTX_BATCH_MAX_OVERRIDES 4
typedef struct otx_batch {
  int32_t num_configs;
  int32_t num_overrides;
  int32_t override_index[OTX_BATCH_MAX_OVERRIDES];
  int32_t tile_size;
  int32_t pad_;
  uint64_t overrides;  /* device otx_surface[num_configs][num_overrides]     */
  uint64_t ray_offset; /* device int64[num_configs + 1], prefix sums         */
  uint64_t tiles;      /* device int32[num_tiles][2]: config, first ray      */
  int64_t num_tiles;
  uint64_t counter;    /* device uint32 work counter (scratch)               */
  uint64_t seed;
  float wl_lo, wl_hi;
  float field_x_half, field_y_half; /* rad */
  float pupil_half;                 /* mm  */
  int32_t image_stride;             /* elements between config images     */
} otx_batch;

/* Learned surrogate of a batch's ray map: a BF16 MLP over 9 inputs (field
 * x, y and pupil x, y normalised by their half ranges, wavelength by the
 * half band about its centre, 4 normalised configuration parameters)
 * predicting the image position as a residual (in out_scale mm units) over
 * a per-configuration quadratic polynomial of the 5 ray inputs, plus a
 * vignetting logit.  No counterpart in the reference. */
#define OTX_SURROGATE_NIN 9    /* network inputs                            */
#define OTX_SURROGATE_LDX 16   /* row pitch of the packed inputs (bf16)     */
#define OTX_SURROGATE_NBASE 21 /* quadratic terms: 1, u_i, u_i u_j (i <= j) */

typedef struct otx_surrogate {
  int32_t num_configs;
  int32_t pad_;
  uint64_t config_inputs; /* device float[num_configs][4], normalised        */
  uint64_t baseline;      /* device float[num_configs][2][NBASE]: x, y (mm)  */
  uint64_t trusted;       /* device uint8[num_configs] or 0 (all trusted):   */
                          /* rays of untrusted configurations are traced    */
  float out_scale;        /* mm per unit of the position outputs            */
  float logit_band;       /* rays with |logit| < logit_band are traced      */
  float pad2_[2];
} otx_surrogate;

/* A BF16 MLP for the fused image simulation: num_hidden SiLU layers of
 * `width` units between num_inputs inputs and num_outputs outputs.  Layer
 * l (0 .. num_hidden; the last is the output layer) has weights w[l], bf16
 * row-major [out x ld[l]] (16-byte aligned rows, ld a multiple of 8) and
 * fp32 biases b[l].  No counterpart in the reference. */
#define OTX_MLP_MAX_HIDDEN 6
typedef struct otx_mlp {
  int32_t num_inputs;
  int32_t num_hidden;
  int32_t width;
  int32_t num_outputs;
  uint64_t w[OTX_MLP_MAX_HIDDEN + 1];
  int32_t ld[OTX_MLP_MAX_HIDDEN + 1];
  int32_t pad_;
  uint64_t b[OTX_MLP_MAX_HIDDEN + 1];
} otx_mlp;

typedef struct otx_launch {
  int32_t rays_per_thread; /* 1, 2 or 4; 0 = library default          */
  int32_t block_size;      /* threads per CTA; 0 = library default     */
  int32_t accumulate;      /* 1: write every surface's rays            */
  int32_t generic_only;    /* 1: never use a shape-specialised kernel  */
} otx_launch;

/* ---- entry points ---------------------------------------------------- */

/* ABI self-description: sizes of the descriptor structs, for binding
 * checks.  `which`: 0 otx_system, 1 otx_surface, 2 otx_rays, 3 otx_grid,
 * 4 otx_image, 5 otx_launch, 6 otx_affine, 7 otx_sensor, 8 otx_layer,
 * 9 otx_stack, 10 otx_periodic_stack, 11 otx_batch, 12 otx_surrogate,
 * 13 otx_mlp. */
int64_t otx_sizeof(int32_t which);
int32_t otx_abi_version(void);
const char* otx_status_string(otx_status s);

/* Trace a ray ensemble through every surface of `sys`.
 * Replaces optika/propagators.py:19-41 (propagate_rays) and :44-73
 * (accumulate_rays, when launch->accumulate), which loop
 * optika/surfaces.py:123-198 (AbstractSurface.propagate_rays) per surface.
 * `in` is in the frame the first surface's `to_local` maps from. */
otx_status otx_trace_rays(const otx_system* sys, const otx_rays* in,
                          const otx_rays* out, const otx_image* image,
                          const otx_launch* launch, void* stream);

/* Build input rays from (wavelength, field, pupil) and trace them.
 * Replaces optika/systems/_sequential.py:791-828 (_calc_rayfunction_input)
 * followed by :836-925 (raytrace) or :927-988 (rayfunction); sensor binning
 * replaces optika/sensors/_sensors.py:92-161 (collect, image histogram). */
otx_status otx_trace_grid(const otx_system* sys, const otx_grid* in,
                          const otx_rays* out, const otx_image* image,
                          const otx_launch* launch, void* stream);

/* otx_trace_grid for grid inputs and ray outputs in HOST memory (page-locked
 * for full speed; pageable works but its copies do not overlap).
 * Replaces the same call chain as otx_trace_grid, for callers whose arrays
 * live on the host as the reference's NumPy arrays do
 * (optika/systems/_sequential.py:791-988 take and return host arrays).
 * The rays pass through the GPU in chunks: the host->device copy of one
 * chunk, the trace of the previous one and the device->host copy of the one
 * before that overlap on two library-owned copy streams and `stream`.
 * Host input strides must be 0 (scalar) or 1.  `out` holds host pointers
 * (accumulate: surface_stride >= count, as in otx_trace_grid); `image`
 * holds DEVICE pointers, accumulated over every chunk.  `workspace` is
 * caller-owned device memory, 256-byte aligned, of workspace_bytes; a
 * smaller workspace than otx_trace_grid_host_workspace() recommends gives
 * smaller chunks (OTX_ERR_SIZE if not even one ray fits).  Stream-ordered:
 * the host outputs are complete when `stream` reaches the point after the
 * call.  The first call on a device creates its copy streams and events. */
otx_status otx_trace_grid_host(const otx_system* sys, const otx_grid* in_host,
                               const otx_rays* out_host, const otx_image* image,
                               const otx_launch* launch, void* workspace,
                               int64_t workspace_bytes, void* stream);
/* Recommended workspace bytes of otx_trace_grid_host for these inputs and
 * outputs (`surfaces` output planes: the system's surface count when
 * accumulating, else 1); -1 for invalid arguments. */
int64_t otx_trace_grid_host_workspace(const otx_grid* in_host, const otx_rays* out_host,
                                      int32_t surfaces);

/* Multilayer reflectivity / transmissivity of `count` samples (float-float
 * transfer matrices).
 * Replaces optika/materials/_multilayers.py:240-532 (multilayer_efficiency).
 * wavelength (nm), cos_incidence (direction), n_ambient (re, im) are float*
 * device arrays with strides (0 = broadcast); stack_index (int32*, may be
 * null = stack 0) selects one of sys->stacks per sample.  Outputs R_s, R_p,
 * T_s, T_p (float*, any may be null). */
otx_status otx_multilayer_efficiency(
    const otx_system* sys, int64_t count, const float* wavelength,
    int64_t stride_wavelength, const float* cos_incidence, int64_t stride_cos,
    const float* n_re, const float* n_im, int64_t stride_n,
    const int32_t* stack_index, float* r_s, float* r_p, float* t_s,
    float* t_p, void* stream);

/* Trace every configuration of a batch in one persistent launch.
 * Replaces optika's broadcasting of a SequentialSystem over configuration
 * axes (optika/_util.py:21-38, shape of every component) in
 * raytrace / rayfunction (optika/systems/_sequential.py:836-988).  Outputs
 * (sensor frame) are indexed ray_offset[config] + ray; images, if given,
 * are per config, image_stride elements apart. */
otx_status otx_trace_batch(const otx_system* base, const otx_batch* batch,
                           const otx_rays* out, const otx_image* image,
                           const otx_launch* launch, void* stream);

/* otx_trace_batch without any allocation by the caller or the library.
 *
 * No counterpart in the reference.  For callers that cannot allocate GPU
 * memory at the point of the call: a host application embedding this
 * library whose device memory belongs to its own allocator, or code that
 * may not allocate (allocation synchronises the device).  They pass only
 * the inputs and outputs of otx_trace_batch; batch->tiles and
 * batch->counter are ignored.  The library builds the tile list itself
 * from batch->ray_offset; batch->num_tiles, the caller's count of work
 * items (sum over configs of ceil(rays / tile_size)), may not exceed
 * OTX_NOALLOC_MAX_TILES (OTX_ERR_SIZE), and work items beyond that
 * capacity are never traced.  Each configuration holds at most 2^31 - 1
 * rays (a larger one is not traced).  The work counter and the tile list
 * live in a file-scope device array of the library (1 MiB, held by every
 * GPU that loads the library until exit), whose address on the current
 * device every call looks up (no allocation); the first call on a device
 * also loads the library's kernels there, so make it before any stream
 * capture.  Every call shares that array and keeps the last call's
 * contents: calls that overlap on the GPU (on concurrent streams) race. */
#define OTX_NOALLOC_MAX_TILES 131000
otx_status otx_trace_batch_noalloc(const otx_system* base, const otx_batch* batch,
                                   const otx_rays* out, const otx_image* image,
                                   const otx_launch* launch, void* stream);

/* Reflectivity / transmissivity of `count` samples over a batch of
 * periodic bilayer mirrors (float-float transfer matrices).  configs is a
 * device array of num_configs entries, config_index (int32*, may be null =
 * config 0) selects one per sample; wavelength (nm) and cos_incidence are
 * float* device arrays with strides (0 = broadcast); the ambient index is
 * n_re + i n_im.  Replaces optika/materials/_multilayers.py:240-532 for
 * PeriodicLayerSequence stacks (optika/materials/_layers.py:611-645). */
otx_status otx_multilayer_periodic(const otx_periodic_stack* configs, int32_t num_configs,
                                   int64_t count, const float* wavelength,
                                   int64_t stride_wavelength, const float* cos_incidence,
                                   int64_t stride_cos, const int32_t* config_index,
                                   float n_re, float n_im, float* r_s, float* r_p,
                                   float* t_s, float* t_p, void* stream);

/* ---- learned surrogate (BF16 MLP on tensor cores) ------------------- */
/* No counterpart in the reference: the surrogate of the ray map is new.   */

#define OTX_EPI_SILU_BF16 0  /* out = bf16(silu(A B^T + bias)), z = bf16(pre)  */
#define OTX_EPI_BIAS_F32 1   /* out = f32(A B^T + bias)                        */
#define OTX_EPI_F32 2        /* out = f32(A B^T)                               */
#define OTX_EPI_DSILU_BF16 3 /* out = bf16(A B^T * silu'(z)), z read           */
#define OTX_EPI_F32_ATOMIC 4 /* out = f32(A B^T), K split over CTAs, summed    */
                             /* by atomics into out (zeroed by the call)       */

/* C[m x n] = epilogue(A B^T + bias): A bf16 [m x k] and B bf16 [n x k],
 * row-major with row pitches lda, ldb (elements, multiples of 8, rows
 * 16-byte aligned); tcgen05 tensor cores, TMA tiles, FP32 accumulation.
 * n <= 256.  z has out's row pitch ldo.  out_t (bf16 epilogues only, may
 * be null) receives the transpose of out with row pitch ldt >= m.  *err
 * (device int) is set if a bounded wait gave up. */
otx_status otx_gemm_bf16(const void* a, int32_t lda, const void* b, int32_t ldb, int32_t m,
                         int32_t n, int32_t k, const float* bias, int32_t epilogue, void* out,
                         int32_t ldo, void* z, void* out_t, int32_t ldt, int32_t* err,
                         void* stream);
/* dz = dy * silu'(z) (dy fp32, z and dz bf16, count elements). */
otx_status otx_silu_backward(const float* dy, const void* z, void* dz, int64_t count,
                             void* stream);
/* out[c][r] = in[r][c] for a bf16 rows x cols matrix. */
otx_status otx_transpose_bf16(const void* in, int32_t rows, int32_t cols, int32_t ldi, void* out,
                              int32_t ldo, void* stream);
/* out[c] = sum over rows of in[r][c] (bf16 in, fp32 out); cols <= 256, the
 * row pitch ldi a multiple of 8 and in 16-byte aligned. */
otx_status otx_colsum_bf16(const void* in, int32_t rows, int32_t cols, int32_t ldi, float* out,
                           void* stream);
/* One Adam step on fp32 master weights w (rows x cols) with moments m, v;
 * writes bf16 copies w16 (row pitch ld16) and, if given, the transpose
 * w16t (row pitch ld16t). */
otx_status otx_adam(float* w, float* m, float* v, const float* grad, int32_t rows, int32_t cols,
                    float lr, float beta1, float beta2, float eps, int32_t step, void* w16,
                    int32_t ld16, void* w16t, int32_t ld16t, void* stream);

/* Network inputs of rays [first, first + count) of a batch (or of rays
 * perm[first + r] when perm is given): x bf16 [count][OTX_SURROGATE_LDX]
 * (columns 9.. zero), x_t (or null) its transpose with row pitch ldt, and
 * aux float4 [count]: with training targets px, py, unvignetted (indexed
 * by batch ray) {residual x, residual y (out_scale units), label, 0};
 * without {baseline x, baseline y (mm), wavelength, configuration}.
 * u (or null) float [count][8] receives the FP32 normalised ray inputs
 * u0..u4 and the configuration, for fitting the baseline. */
otx_status otx_surrogate_pack(const otx_batch* batch, const otx_surrogate* sg, int64_t first,
                              int64_t count, const int64_t* perm, const float* px,
                              const float* py, const uint8_t* unvignetted, void* x, void* x_t,
                              int32_t ldt, float* aux, float* u, void* stream);
/* Training loss of network outputs y (fp32 [count][ldy]: residual x, y,
 * logit) against aux targets: w_pos * sum(label * |dr|^2) + w_cls * sum(BCE),
 * both times norm.  Writes dL/dy as bf16 [count][8] (columns 3.. zero) and
 * its transpose dy_t [3][ldt]; adds {sum label |dr|^2, sum BCE, sum label,
 * correct classifications} into sums[4]. */
otx_status otx_surrogate_loss(const float* y, int32_t ldy, const float* aux, int64_t count,
                              float w_pos, float w_cls, float norm, void* dy, void* dy_t,
                              int32_t ldt, float* sums, void* stream);
/* Image simulation of rays [first, first + count) of a batch from network
 * outputs y and packed aux: rays of trusted configurations with |logit| >=
 * logit_band land at baseline + out_scale * y (if logit > 0); the others
 * are traced through base (with the batch's overrides) in the same kernel.
 * Adds into the per-configuration images and stats[4] = {rays, traced,
 * binned by the network, binned by the trace}. */
otx_status otx_surrogate_image(const otx_system* base, const otx_batch* batch,
                               const otx_surrogate* sg, int64_t first, int64_t count,
                               const float* y, int32_t ldy, const float* aux,
                               const otx_image* image, unsigned long long* stats, void* stream);

/* Image simulation of rays [first, first + count) of a batch in one
 * persistent tensor-core kernel: the rays are generated, the network (9
 * inputs, hidden width 256, 3 outputs) runs layer after layer with its
 * activations kept in shared memory and its accumulators in TMEM, and rays
 * of trusted configurations with |logit| >= logit_band land at baseline +
 * out_scale * output (binned if logit > 0); every other ray is queued and
 * traced through base (with the batch's overrides) by a second kernel.
 * Same results as otx_surrogate_pack + otx_gemm_bf16 per layer +
 * otx_surrogate_image up to FP32 rounding.  `predict` (device float4
 * [count], 16-byte aligned, or null) receives each ray's predicted
 * position (mm) and logit; with predict and no image nothing is binned,
 * queued or traced.  `workspace` (device, 256-byte aligned,
 * otx_surrogate_image_fused_workspace() bytes) holds the queue.  Adds into
 * the per-configuration images and stats[4] = {rays, traced, binned by the
 * network, binned by the trace}; *err (device int) is set if a bounded wait
 * gave up.  No counterpart in the reference. */
otx_status otx_surrogate_image_fused(const otx_system* base, const otx_batch* batch,
                                     const otx_surrogate* sg, const otx_mlp* net,
                                     int64_t first, int64_t count, const otx_image* image,
                                     float* predict, void* workspace, int64_t workspace_bytes,
                                     unsigned long long* stats, int32_t* err, void* stream);
/* Workspace bytes of otx_surrogate_image_fused for `count` rays of this
 * batch and network; -1 for invalid arguments. */
int64_t otx_surrogate_image_fused_workspace(const otx_batch* batch, const otx_mlp* net,
                                            int64_t count);

/* Bin rays given in the sensor's local frame into count and flux images.
 * Replaces optika/sensors/_sensors.py:92-161 (ImagingSensor.collect, the
 * intensity-weighted na.histogram of position.xy and wavelength).  Reads
 * px, py, wavelength (when wavelength bins are set), intensity and
 * unvignetted of `rays`. */
otx_status otx_collect(const otx_sensor* sensor, const otx_rays* rays,
                       const otx_image* image, void* stream);

/* Newton solve of the stop rays, one thread per ray (a pair of stop
 * boundary points at one wavelength).
 * Replaces the Newton loop of optika/systems/_sequential.py:396-693
 * (_calc_rayfunction_stops_only, its _ray_error at :363-394): the free
 * component (x, y) of each ray at the first stop -- its direction, z then
 * sqrt(1 - x^2 - y^2), or with `free_position` its position, z the sag of
 * first_sag->surfaces[0] -- is moved until the ray, traced through `sub`
 * (the surfaces after the first stop, input in the system frame, output
 * in sub's final_to_output frame) and mapped by `to_last` (3 x 4 affine,
 * float64, row-major) lands on (target_x, target_y): the point's or, with
 * `target_direction`, the direction's first two components.  Each
 * iteration takes a forward-difference Jacobian with `step`; a ray whose
 * residual falls below `tolerance` takes `polish_steps` more steps.
 * position and direction are device float64 [3][count] arrays (in: the
 * starting rays; out: the solved ones); wavelength, target_x, target_y
 * device float64 [count]; status device int32 [count]: the iteration at
 * which the ray finished, -1 if it did not within max_iterations. */
typedef struct otx_stop_solve {
  int64_t count;
  int32_t free_position;    /* 1: the ray's position on the first stop is free */
  int32_t target_direction; /* 1: the target is the direction at the last stop */
  int32_t max_iterations;
  int32_t polish_steps;
  double step;
  double tolerance;
  double to_last[12];
  uint64_t position, direction, wavelength, target_x, target_y, status;
} otx_stop_solve;
otx_status otx_stop_newton(const otx_system* sub, const otx_system* first_sag,
                           const otx_stop_solve* solve, void* stream);

/* Evaluate the sag of sys->surfaces[0] at `in` positions.
 * mode 0: sag z(x, y) into out->pz   (optika/sags/_abc.py:48-62 __call__)
 * mode 1: unit normal into out->d*   (optika/sags/_abc.py:64-75 normal)
 * mode 2: intercept of the rays (in->p*, in->d*) into out->p*
 *         (optika/sags/_abc.py:76-107 intercept and its overrides). */
otx_status otx_sag_eval(const otx_system* sys, int32_t mode, const otx_rays* in,
                        const otx_rays* out, void* stream);

/* Cells of a scene for SequentialSystem.image (optika/systems/
 * _sequential.py:1002-1086 _rayfunction_from_vertices): one ray per cell
 * of the (wavelength, field x, field y, pupil x, pupil y) vertex grid, at a
 * uniformly drawn point of the cell (or its centre), carrying the cell's
 * flux.  Field and pupil vertices are given at every wavelength vertex
 * (normalised coordinates are denormalised per wavelength by the stop
 * solver); inside a cell they are interpolated with the same wavelength
 * weight as the wavelength itself.  All tables are float device arrays. */
typedef struct otx_cells {
  uint64_t wavelength;   /* [nw + 1] vertices (nm)                          */
  uint64_t field_x;      /* [nw + 1][nfx + 1]                                */
  uint64_t field_y;      /* [nw + 1][nfy + 1]                                */
  uint64_t pupil_x;      /* [nw + 1][npx + 1]                                */
  uint64_t pupil_y;      /* [nw + 1][npy + 1]                                */
  uint64_t weight;       /* [nw][nfx][nfy] radiance x wavelength width x
                            field cell area (solid angle or area)            */
  uint64_t weight_pupil; /* [nw][npx][npy] pupil cell area (or solid angle) */
  int32_t nw, nfx, nfy, npx, npy;
  int32_t random;        /* 1: uniform point of each cell; 0: its centre     */
  uint64_t seed;         /* Philox key of the draws                          */
} otx_cells;

/* Input rays of cells [first, first + count) (ray index = ((((iw nfx + ifx)
 * nfy + ify) npx + ipx) npy + ipy) into out->wavelength, field_x, field_y,
 * pupil_x, pupil_y and intensity (each a float array of `count` entries;
 * out's strides are ignored).  The rays then go through otx_trace_grid
 * with sensor binning, as rayfunction does in the reference. */
otx_status otx_cell_rays(const otx_cells* cells, int64_t first, int64_t count,
                         const otx_grid* out, void* stream);

/* Cells [first, first + count) traced with their rays generated in the
 * trace kernel (the rays of otx_cell_rays, never written to memory) and
 * binned into `image` (required: it is the only output).  Replaces, fused,
 * the cell sampling of SequentialSystem._rayfunction_from_vertices
 * (optika/systems/_sequential.py:1002-1086) and the rayfunction and
 * sensor.measure calls of SequentialSystem.image (:1088-1206).  The
 * system's input_mode (grid at infinity or finite) tells how a cell's
 * field and pupil coordinates make its ray. */
otx_status otx_trace_cells(const otx_system* sys, const otx_cells* cells, int64_t first,
                           int64_t count, const otx_image* image, const otx_launch* launch,
                           void* stream);

/* Detector exposure of an ideal sensor (optika/sensors/_sensors.py:173-252
 * expose; optika/sensors/materials/_materials.py:1576-1598 signal):
 * electrons[i] = Poisson(scale photons[i]) + read_noise N(0, 1) when
 * `noise` is set, scale photons[i] otherwise.  Poisson variates by
 * transformed rejection (Hormann 1993) for means >= 10 and by the
 * multiplication method below; normal variates by Box-Muller; one Philox
 * stream per pixel keyed by `seed`. */
otx_status otx_expose(const float* photons, float* electrons, int64_t count, float scale,
                      float read_noise, int32_t noise, uint64_t seed, void* stream);

/* Masked reductions of traced rays over the pupil, the first step of the
 * reference's calibration fits (optika/systems/_sequential.py:1208-1512:
 * distortion, vignetting, area_effective).  The rays are `groups` runs of
 * `per_group` consecutive rays (one run per wavelength and field point,
 * the pupil fastest).  For each group g, sums[g * 6 + k] receives
 *   k = 0: the number of unvignetted rays,
 *       1, 2: the sums of px, py over the unvignetted rays,
 *       3, 4: the sums of px, py over all rays,
 *       5: the sum of intensity over the unvignetted rays
 * (double precision).  Reads px, py, intensity (1 if null) and
 * unvignetted (all if null) of `rays`; rays->count must be
 * groups * per_group. */
otx_status otx_pupil_reduce(const otx_rays* rays, int64_t groups, int64_t per_group,
                            double* sums, void* stream);

/* Evaluate the rulings of sys->surfaces[0] for rays at the surface (in the
 * surface frame) with the sag normals `normal` (normal->dx, dy, dz; the
 * rays' direction in rays->d*, position in rays->p*, wavelength in nm).
 * mode 0: groove efficiency into efficiency[count]
 *         (optika/rulings/_rulings.py:207-222 efficiency and its models)
 * mode 1: effective incident direction into out->d*
 *         (optika/rulings/_rulings.py:170-204 incident_effective).
 * Surfaces without rulings return OTX_ERR_INVALID. */
otx_status otx_rulings_eval(const otx_system* sys, int32_t mode, const otx_rays* rays,
                            const otx_rays* normal, float* efficiency, const otx_rays* out,
                            void* stream);

#ifdef __cplusplus
}
#endif

#endif /* OPTIKA_GB300_H */
