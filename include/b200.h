/* b200: the GB300 device module's C ABI for the OSPRay render hot path.
 *
 * Plain C: opaque handles, host or device pointers with explicit sizes, and
 * an int status on every call (0 = success, otherwise an OSPError value;
 * ospray/include/ospray/OSPEnums.h OSPError).  No call throws.  The message
 * of the last failure on a device is returned by b200_device_last_error
 * (ospDeviceGetLastErrorMsg, ospray/api/API.cpp:28-66).
 *
 * Each group of entry points names the reference interface it replaces.
 * Coordinates, ray layouts, identifier conventions and framebuffer formats
 * are those of the reference: triangle u/v with P = (1-u-v) v0 + u v1 + v v2,
 * RGBA32F colour, images with row 0 at the bottom, invalid IDs = 0xffffffff.
 */
#ifndef B200_H
#define B200_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define B200_VERSION_MAJOR 3
#define B200_VERSION_MINOR 3
#define B200_VERSION_PATCH 0

/* status codes = OSPError (ospray/include/ospray/OSPEnums.h) */
enum {
  B200_NO_ERROR = 0,
  B200_UNKNOWN_ERROR = 1,
  B200_INVALID_ARGUMENT = 2,
  B200_INVALID_OPERATION = 3,
  B200_OUT_OF_MEMORY = 4,
  B200_UNSUPPORTED_CPU = 5,
  B200_VERSION_MISMATCH = 6
};

typedef struct b200_device_t *b200_device;
typedef struct b200_scene_t *b200_scene;
typedef struct b200_frame_t *b200_frame;

/* ---- device (replaces ISPCDevice construction/commit,
 *      modules/cpu/ISPCDevice.cpp:207-326, and ospDeviceGetLastErrorMsg) */
int b200_device_create(int cuda_device, b200_device *out);
int b200_device_release(b200_device dev);
const char *b200_device_last_error(b200_device dev);
/* the CUDA stream (cudaStream_t) all work of this device is ordered on */
void *b200_device_stream(b200_device dev);
int b200_device_sync(b200_device dev);

/* Live kernel timing (no reference counterpart; the reference reports frame
 * times only, ospray/include/ospray/ospray.h:335 ospGetTaskDuration).  While enabled, the
 * renderers record a pair of CUDA events on the launch stream around every
 * launch of their hot kernels; b200_kernel_timing_read waits for them and
 * returns per kind (0 closest-hit trace, 1 shadow trace, 2 path-tracer
 * shade, 3 AO frame kernel, 4 SciVis volume kernel) the summed device
 * milliseconds and launch counts, optionally resetting them. */
int b200_kernel_timing(b200_device dev, int enable);
int b200_kernel_timing_read(b200_device dev, double *ms, int64_t *launches, int n, int reset);

/* ---- completion events on the device stream: what an OSPFuture waits on
 *      (ospRenderFrame / ospIsReady / ospWait / ospGetTaskDuration,
 *      ospray/include/ospray/ospray.h:315-336; the reference's future is a
 *      task-system future, render/RenderingFuture.h:55-87).  An event marks
 *      the point of the stream where it was recorded. */
typedef struct b200_event_t *b200_event;
int b200_event_record(b200_device dev, b200_event *out);
/* 1 when all work before the event has finished, 0 if not, < 0 on error */
int b200_event_query(b200_event ev);
int b200_event_wait(b200_event ev);
/* milliseconds between two completed events of one device */
float b200_event_elapsed_ms(b200_event start, b200_event end);
int b200_event_release(b200_event ev);

/* ---- world: geometry upload and acceleration-structure build
 *      (Mesh::commit modules/cpu/geometry/Mesh.cpp:37-204,
 *       Spheres::commit geometry/Spheres.cpp:46-106,
 *       Group::commit common/Group.cpp:69-143,
 *       World::commit common/World.cpp:70-188).
 * Host arrays are copied to the device at the call; the caller keeps
 * ownership of its memory. */
int b200_scene_create(b200_device dev, b200_scene *out);
int b200_scene_release(b200_scene scene);
/* vertex: nverts x 3 float; index: ntris x 3 uint32 (vec3ui) */
int b200_scene_add_mesh(b200_scene scene, const float *vertex, int64_t nverts, const uint32_t *index,
                        int64_t ntris, int *geom_out);
/* Quad mesh (Mesh::commit with a vec4ui "index", Mesh.cpp:114-145;
 * QuadMesh_postIntersect geometry/Mesh.ispc:67-176): index nquads x 4
 * uint32.  A quad (v0, v1, v2, v3) is intersected as the triangles
 * (v0, v1, v3) and (v2, v3, v1), Embree's quad decomposition; a hit reports
 * the quad's index as primID, and the epsilon is taken over its 4 vertices.
 * A triangle given as a quad with v2 == v3 adds a degenerate half that is
 * never hit. */
int b200_scene_add_quad_mesh(b200_scene scene, const float *vertex, int64_t nverts, const uint32_t *index,
                             int64_t nquads, int *geom_out);
/* Boxes (Boxes::commit geometry/Boxes.cpp:33-46, "box" data of box3f):
 * boxes n x 6 float (lower xyz, upper xyz).  Each box is traced as its 12
 * face triangles, which report the box's index as primID; a ray hits the
 * first face in [tnear, tfar] (the exit face when it starts inside, as
 * intersectBox with filterIntersectionBoth, common/Intersect.ih:195-223),
 * the normal is the face's, and no geometry epsilon is added
 * (Boxes_postIntersect). */
int b200_scene_add_boxes(b200_scene scene, const float *boxes, int64_t n, int *geom_out);
/* spheres: n x 4 float (center xyz, radius), OSP_SPHERE */
int b200_scene_add_spheres(b200_scene scene, const float *spheres, int64_t n, int *geom_out);
/* discs (Spheres::commit "type", geometry/Spheres.cpp:21-22,43-54): n x 4
 * float (center xyz, radius); normals null: OSP_DISC, discs facing the ray;
 * normals n x 3 float: OSP_ORIENTED_DISC ("sphere.normal") */
int b200_scene_add_discs(b200_scene scene, const float *discs, int64_t n, const float *normals, int *geom_out);
/* planes (Planes::commit geometry/Planes.cpp, Planes.ispc): n x 4 float
 * "plane.coefficients" (a, b, c, d: the plane a x + b y + c z = d, as the
 * reference's intersectPlane), bounds null (unbounded, +-1e18) or n x 6 float
 * "plane.bounds" (lower xyz, upper xyz) */
int b200_scene_add_planes(b200_scene scene, const float *coeffs, int64_t n, const float *bounds, int *geom_out);
/* Per-vertex attributes of a triangle mesh (Mesh::commit "vertex.normal",
 * "vertex.color", "vertex.texcoord", geometry/Mesh.cpp:37-204;
 * TriangleMesh_postIntersect geometry/Mesh.ispc:178-276), each nverts x
 * (3, 4, 2) floats or null; call before the scene's commit.  Normals give the
 * interpolated shading normal, colours multiply the path tracer's material
 * colours (alpha the OBJ d), texture coordinates address material textures
 * and define the shading tangents (without them textures see the hit's
 * barycentric u, v).  Used by the path tracer. */
int b200_scene_set_mesh_attributes(b200_scene scene, int geom, const float *normal, const float *color,
                                   const float *texcoord);
/* one (instance, geometric model) pair: geometry `geom` placed by the
 * row-major 3x4 affine `xfm` (null = identity), reported as instID/geomID;
 * material_id indexes the renderer's material list (or -1 for none) */
int b200_scene_add_instance(b200_scene scene, int geom, uint32_t inst_id, uint32_t geom_id, const float *xfm,
                            int material_id);
/* A motion-blurred (instance, geometric model) pair (Instance "motion.transform"
 * and "time", MotionTransform::readParams common/MotionTransform.cpp:10-66):
 * nkeys >= 2 row-major 3x4 transforms `xfms` at times evenly spaced over
 * [t0, t1] (t1 < t0 is raised to t0).  A ray at time t sees the geometry
 * under the two keys around t blended component-wise, (1 - f) A + f B, the
 * interpolation Embree applies to key-framed instance matrices; times
 * outside [t0, t1] take the end keys.  The TLAS bounds the instance by the
 * union of its keys' boxes, which contains every blend. */
int b200_scene_add_instance_motion(b200_scene scene, int geom, uint32_t inst_id, uint32_t geom_id,
                                   const float *xfms, int nkeys, float t0, float t1, int material_id);
/* build quality of the commits that follow (Group/World "dynamicScene",
 * common/Group.cpp:17-31 selects Embree's low build quality): dynamic != 0
 * builds the plain LBVH hierarchy (fastest build); the default splits the
 * Morton-ordered primitive ranges by binned SAH */
int b200_scene_set_dynamic(b200_scene scene, int dynamic);
/* builds every BLAS not yet built and the TLAS */
int b200_scene_commit(b200_scene scene);
/* world bounds after commit: lo xyz, hi xyz */
int b200_scene_bounds(b200_scene scene, float *box6);
/* BVH statistics after commit: [nodes, primitives] summed over BLASes, TLAS nodes */
int b200_scene_stats(b200_scene scene, int64_t *stats3);

/* ---- ray queries (rtcIntersectV / rtcOccludedV behind traceGeometryRay and
 *      isOccluded, modules/cpu/common/World.ih:29-52,311-380).
 * Device pointers.  rays: n x 8 float (org xyz, tnear, dir xyz, tfar).
 * occlusion == 0: hit_f n x 6 float (t, u, v, Ng xyz object space; t = inf
 *   on a miss), hit_id n x 3 uint32 (primID, geomID, instID).
 * occlusion != 0: hit_f[6 i] = 1 if any hit in [tnear, tfar] else 0.
 * stream: cudaStream_t or null for the device stream. */
int b200_trace(b200_scene scene, const float *rays, int64_t n, int occlusion, float *hit_f, uint32_t *hit_id,
               void *stream);

/* ---- camera (PerspectiveCamera::commit, modules/cpu/camera/PerspectiveCamera.cpp:30-117) */
/* type: B200_CAMERA_PERSPECTIVE (PerspectiveCamera, fovy / aspect),
 * B200_CAMERA_ORTHOGRAPHIC (OrthographicCamera::commit
 * camera/OrthographicCamera.cpp:25-50: `height` of the image plane and
 * aspect) or B200_CAMERA_PANORAMIC (PanoramicCamera, equirectangular; no
 * stereo).
 * Shutter (Camera::commit camera/Camera.cpp:44-52,100-119 and
 * Camera_shutterTime camera/Camera.ih:33-42): "shutter" [lower, upper]
 * clamped to [0, 1], "shutterType" (OSPShutterType: 0 global, 1 rolling
 * right, 2 rolling left, 3 rolling down, 4 rolling up) and
 * "rollingShutterDuration".  The path tracer draws each camera sample's
 * time from its own sample stream when the shutter is open (global: upper >
 * lower; rolling: duration > 0), else takes the shutter time of 0.5; the AO
 * and SciVis renderers always take 0.5.  The ray's time places
 * motion-blurred instances (b200_scene_add_instance_motion).  A
 * zero-initialised shutter traces every ray at time 0; OSPRay's default is
 * [0.5, 0.5].  The path tracer draws the lens sample of a perspective
 * camera with an aperture from its sample stream; AO and SciVis use a
 * pinhole (RendererRenderTaskFn.inl:61-63).  "imageStart" / "imageEnd"
 * select the sub-image the frame covers (Camera_subRegion,
 * camera/Camera.ih:28-31); an all-zero pair is the whole image [0, 1]^2.
 * "stereoMode" (OSPStereoMode: 0 none, 1 left, 2 right, 3 side by side, 4
 * top / bottom, left eye at the top) with "interpupillaryDistance" applies
 * to perspective and panoramic cameras (PerspectiveCamera.cpp:37-91,
 * PanoramicCamera.cpp:45-52).  Camera motion is not built. */
enum { B200_CAMERA_PERSPECTIVE = 0, B200_CAMERA_ORTHOGRAPHIC = 1, B200_CAMERA_PANORAMIC = 2 };
typedef struct {
  float position[3], direction[3], up[3];
  float fovy, aspect, nearClip;
  int type;     /* default 0: perspective */
  float height; /* orthographic: image-plane height (OSPRay default 1) */
  float shutter[2];
  int shutterType;
  float rollingShutterDuration;
  /* perspective: depth of field ("apertureRadius", "focusDistance"; a zero
   * radius is a pinhole) and "architectural" (the image plane parallel to
   * up) as PerspectiveCamera::commit camera/PerspectiveCamera.cpp:30-117 */
  float apertureRadius, focusDistance;
  int architectural;
  float imageStart[2], imageEnd[2];
  int stereoMode;
  float interpupillaryDistance;
} b200_camera_desc;

/* ---- framebuffer (LocalFrameBuffer, modules/cpu/fb/LocalFB.cpp:23-226;
 *      formats OSPFrameBufferFormat and channels OSPFrameBufferChannel,
 *      ospray/include/ospray/OSPEnums.h:240-266) */
enum { B200_FB_NONE = 0, B200_FB_RGBA8 = 1, B200_FB_SRGBA = 2, B200_FB_RGBA32F = 3 };
enum {
  B200_FB_COLOR = 1 << 0,
  B200_FB_DEPTH = 1 << 1,
  B200_FB_ACCUM = 1 << 2,
  B200_FB_VARIANCE = 1 << 3,
  B200_FB_NORMAL = 1 << 4,
  B200_FB_ALBEDO = 1 << 5,
  B200_FB_ID_PRIMITIVE = 1 << 6,
  B200_FB_ID_OBJECT = 1 << 7,
  B200_FB_ID_INSTANCE = 1 << 8
};
/* ospNewFrameBuffer(width, height, format, channels).  The colour channel
 * always accumulates in RGBA32F on the device; after every render the
 * frame's post-processing step (tonemapper, if set, then conversion to
 * `format`) writes the mapped colour, as LocalFrameBuffer::postProcess does
 * (fb/LocalFB.cpp:459-477). */
int b200_frame_create(b200_device dev, int width, int height, int format, uint32_t channels, b200_frame *out);
int b200_frame_release(b200_frame fb);
/* ospResetAccumulation: frameID back to 0 */
int b200_frame_reset(b200_frame fb);
int b200_frame_id(b200_frame fb);
/* device pointer of one channel as ospMapFrameBuffer would return it:
 * COLOR = the converted colour (RGBA8/SRGBA: W*H uint32, RGBA32F: W*H*4
 * float; FB_NONE: the raw accumulation buffer), DEPTH float, NORMAL/ALBEDO
 * float3 (accumulated like the colour: AO and SciVis the first hit's shading
 * normal and surface albedo, or on a miss the ray direction / background
 * (AO); the path tracer the first vertex's normal and BSDF albedo; batched
 * renders write 0), IDs uint32, VARIANCE float4.  ACCUM gives the accumulated RGBA32F
 * colour before post-processing (an addition: the reference cannot map it).
 * Rows bottom-up. */
void *b200_frame_channel(b200_frame fb, uint32_t channel);
/* bytes of one mapped channel */
size_t b200_frame_channel_bytes(b200_frame fb, uint32_t channel);
/* ospMapFrameBuffer: copies a channel to host memory (waits for the device) */
int b200_frame_read(b200_frame fb, uint32_t channel, void *host_dst, size_t bytes);
/* ospMapFrameBuffer into page-locked host memory owned by the frame (one
 * buffer per channel, allocated at its first map, freed with the frame):
 * copies the channel there, waits, and returns the pointer in *out.  The
 * contents stay valid until the next b200_frame_map of the same channel or
 * the frame's release. */
int b200_frame_map(b200_frame fb, uint32_t channel, const void **out);

/* ---- tonemapper frame operation (ToneMapper::commit
 *      fb/frame_ops/ToneMapper.cpp:16-51, ToneMapper_kernel
 *      fb/frame_ops/ToneMapper.ispc:12-41; parameter defaults are the ACES
 *      filmic fit: exposure 1, contrast 1.6773, shoulder 0.9714, midIn 0.18,
 *      midOut 0.18, hdrMax 11.0785, acesColor 1).  Setting it is
 *      ospSetObjectAsData(fb, "imageOperation", ...) + ospCommit(fb); a null
 *      `tm` removes it.  It applies from the next render on. */
typedef struct {
  float exposure, contrast, shoulder, midIn, midOut, hdrMax;
  int acesColor;
} b200_tonemapper;
/* fills `tm` with the defaults above */
void b200_tonemapper_defaults(b200_tonemapper *tm);

/* ospGetVariance: the framebuffer's error estimate (needs the VARIANCE
 * channel; updated after every odd frame): per 8x8 task the mean over its
 * pixels of |colour - odd-frame colour|_1 / sqrt(r + g + b + 1 - a) x 64;
 * the mean of the tasks' errors at or above `threshold`, else the largest;
 * inf before the first estimate (fb/frame_ops/Variance.ispc:11-49,
 * Variance.cpp:32-46).  Synchronous.  Batched renders do not update it. */
int b200_frame_variance(b200_frame fb, float threshold, float *out);

/* Adaptive accumulation: the renderer's "varianceThreshold"
 * (Renderer::commit render/Renderer.cpp:44), applied by later render calls
 * on this framebuffer (LocalTiledLoadBalancer::renderFrame
 * render/LoadBalancer.cpp:15-30 with LocalFrameBuffer::getRenderTaskIDs
 * fb/LocalFB.cpp:238-260).  With a threshold > 0, a VARIANCE channel and a
 * frame ID >= max(2, 16 / pixelSamples), a render call renders only the
 * 8x8 tasks whose last error estimate exceeds the threshold; the other
 * pixels keep their accumulated values.  0 (the default) renders every task.
 * A non-finite value is refused.  Batched renders ignore it. */
int b200_frame_set_variance_threshold(b200_frame fb, float varianceThreshold);

/* image error of a framebuffer's accumulated colour against a reference
 * framebuffer of the same size: relMSE = mean over pixels and rgb of
 * (x - r)^2 / (r^2 + 0.01).  Synchronous. */
int b200_frame_relmse(b200_frame fb, b200_frame reference, double *out);
/* the same over the pixels whose first hit in the reference is geometry
 * (finite reference DEPTH; the reference needs that channel), so pixels of
 * constant background radiance do not dilute the mean; npix (may be null)
 * receives their count.  Synchronous. */
int b200_frame_relmse_hits(b200_frame fb, b200_frame reference, double *out, int64_t *npix);
int b200_frame_set_tonemapper(b200_frame fb, const b200_tonemapper *tm);

/* ---- AO renderer (AORenderer::commit modules/cpu/render/ao/AORenderer.cpp:26-35,
 *      AORenderer_renderSample render/ao/AORenderer.ispc:23-149).
 * One call renders one frame and accumulates it into fb (ospRenderFrame). */
enum { B200_PF_POINT = 0, B200_PF_BOX = 1, B200_PF_GAUSS = 2, B200_PF_MITCHELL = 3, B200_PF_BLACKMAN_HARRIS = 4 };
typedef struct {
  int pixelSamples;  /* spp, >= 1 */
  int aoSamples;
  float aoDistance;  /* aoRadius */
  float aoIntensity;
  float backgroundColor[4];
  int pixelFilter;   /* B200_PF_* */
  int collectStats;  /* nonzero: count rays / node visits / primitive tests */
  float volumeSamplingRate; /* the scene's volume, composited in front of each layer (render/ao/volumes.ispc);
                               <= 0: 1 */
  /* the renderer's "map_backplate" and "map_maxDepth" (Renderer_getBackground /
   * Renderer_getMaxDepth render/Renderer.ispc:19-40), both looked up at the
   * pixel centre; null: backgroundColor / no depth limit */
  struct b200_texture_t *backplate;
  struct b200_texture_t *maxDepth;
  float mipMapBias;
  /* surface colour and opacity (getSurfaceColor render/ao/surfaces.ispc:
   * 17-42): obj materials' kd, d and map_kd times the vertex colour; a ray
   * continues through surfaces that are not opaque.  Indexed by the
   * instances' material_id; null / 0: white, opaque surfaces */
  const struct b200_scivis_material_t *materials;
  int nmaterials;
} b200_ao_params;

/* ---- lights of the world (QuadLight::commit lights/QuadLight.cpp:68-108,
 *      AmbientLight::commit lights/AmbientLight.cpp:40-60, Light::commit
 *      lights/Light.cpp:22-35).  radiance = color * intensity (the default
 *      intensityQuantity of both).  The list order is the light index order of
 *      the path tracer's light CDF (render/pathtracer/PathTracerData.cpp:32-82). */
enum { B200_LIGHT_QUAD = 0, B200_LIGHT_AMBIENT = 1, B200_LIGHT_DISTANT = 2, B200_LIGHT_SPHERE = 3, B200_LIGHT_SPOT = 4 };
/* distant (DirectionalLight::commit lights/DirectionalLight.cpp:77-105):
 *   `direction` the light travels, `angularDiameter` in degrees (clamped to
 *   [0, 180]); irradiance = color * intensity (intensityQuantity IRRADIANCE).
 * sphere (PointLight::commit lights/PointLight.cpp:68-121): `position`,
 *   `radius` (0: a point light); radiative intensity = color * intensity
 *   (intensityQuantity INTENSITY), radiance = that / (pi radius^2).
 * spot (SpotLight::commit lights/SpotLight.cpp:76-140, no intensity
 *   distribution): `position`, `direction` it points to, `openingAngle`
 *   (degrees, clamped to [0, 360]), `penumbraAngle` (clamped to half the
 *   opening), `radius` / `innerRadius` of its emitting ring (0: a point);
 *   radiative intensity = color * intensity, radiance = that / ring area.
 * Unused fields are ignored; zero-initialise the struct. */
typedef struct {
  int type;
  int visible;
  float position[3], edge1[3], edge2[3];
  float color[3];
  float intensity;
  float direction[3];
  float angularDiameter;
  float radius;
  float openingAngle, penumbraAngle, innerRadius;
} b200_light;
int b200_scene_set_lights(b200_scene scene, const b200_light *lights, int n);

/* ---- 2D textures (Texture2D::commit texture/Texture2D.cpp:42-146,
 *      Texture2D_get texture/Texture2D.ispc:130-164).
 * data: width x height texels of `format` (OSPTextureFormat values: RGBA8,
 * SRGBA, RGBA32F, RGB8, SRGB, RGB32F, R8, R32F, L8, RA8, LA8, RGBA16, RGB16,
 * RA16, R16, RA32F; the half-float formats are refused), rows from the
 * bottom, copied at the call; filter OSPTextureFilter (0 linear, 1 nearest);
 * wrap modes OSPTextureWrapMode per axis (0 repeat, 1 mirrored repeat,
 * 2 clamp to edge).  mipmaps != 0 generates the MIP chain on the device
 * (MipMap_generate, texture/MipMapGeneration.ispc) and lookups then pick the
 * level from the ray cone's footprint.  A texture must outlive the materials
 * and renders that use it. */
typedef struct b200_texture_t *b200_texture;
int b200_texture_create(b200_device dev, int width, int height, int format, int filter, int wrapS, int wrapT,
                        int mipmaps, const void *data, b200_texture *out);
int b200_texture_release(b200_texture tex);
/* number of levels (1 + MIP levels) */
int b200_texture_levels(b200_texture tex);
/* copies level `level` (max(w >> level, 1) x max(h >> level, 1) texels of the
 * texture's format) into host memory `dst` of `bytes` bytes */
int b200_texture_read_level(b200_texture tex, int level, void *dst, size_t bytes);
/* Texture2D_get at n texture coordinates (st: 2 floats each, host memory)
 * with per-lookup pixel footprints (0: level 0); out: n x RGBA floats */
int b200_texture_sample(b200_texture tex, int64_t n, const float *st, const float *footprint, float *out);

/* ---- path tracer (PathTracer::commit render/pathtracer/PathTracer.cpp:29-51,
 *      PathTracer_renderPixel render/pathtracer/PathTracer.ispc:75-216).
 * material_id of an instance (b200_scene_add_instance) indexes `materials`.
 * A material is one of the reference's material types with the parameters
 * below; fill a struct with b200_material_defaults first (the reference's
 * parameter defaults), then set what differs.
 *   B200_MATERIAL_PRINCIPLED  (render/materials/Principled.ispc:81-455,
 *     Principled.cpp:37-79): baseColor, roughness, metallic, opacity (the
 *     cut-out: a specular transmission lobe of importance 1 - opacity, and
 *     shadow rays pass with transparency 1 - opacity), specular (the
 *     dielectric coating's weight), ior (the coating's index), diffuse (the
 *     substrate's weight), edgeColor (the conductor's edge tint) and
 *     specularMetallic; roughness 0 gives smooth (Dirac) coating and
 *     conductor lobes over a Lambert substrate.  Transmission, thin, coat,
 *     sheen, backlight and emission keep their defaults (off).
 *   B200_MATERIAL_OBJ  (render/materials/OBJ.ispc:29-126, OBJ.cpp:28-65):
 *     kd = baseColor, ks, ns, d = opacity, tf: Lambert (kd d) + Blinn
 *     specular (ks d, exponent ns) + specular transmission (tf d + 1 - d);
 *     kd + ks + tf above 1 is scaled down to 1 as OBJ::commit does.
 *   B200_MATERIAL_METAL  (render/materials/Metal.ispc:16-48, Metal.cpp:27-70):
 *     complex index of refraction eta + i k per RGB channel (default
 *     aluminium) and roughness: a specular conductor at roughness 0, else a
 *     GGX microfacet conductor.
 *   B200_MATERIAL_GLASS  (render/materials/Glass.ispc:16-60, Glass.cpp:27-50):
 *     eta[0] = etaInside, eta[1] = etaOutside, attenuationColor and
 *     attenuationDistance of the inside medium: a smooth dielectric; paths
 *     track the medium they travel in and attenuate by Beer's law.
 *   B200_MATERIAL_THINGLASS  (render/materials/ThinGlass.ispc:16-70,
 *     ThinGlass.cpp:27-45): eta[0] = eta, attenuationColor,
 *     attenuationDistance, thickness: a thin dielectric slab. */
enum {
  B200_MATERIAL_PRINCIPLED = 0,
  B200_MATERIAL_OBJ = 1,
  B200_MATERIAL_METAL = 2,
  B200_MATERIAL_GLASS = 3,
  B200_MATERIAL_THINGLASS = 4
};
typedef struct {
  float baseColor[3];  /* principled baseColor; obj kd */
  float roughness;     /* principled, metal */
  float metallic;      /* principled */
  int type;            /* B200_MATERIAL_* */
  float opacity;       /* principled opacity; obj d */
  float ks[3], ns;     /* obj */
  float tf[3];         /* obj transmission filter */
  float eta[3], k[3];  /* metal: eta + i k per RGB; glass: etaInside, etaOutside; thinGlass: eta */
  float attenuationColor[3];
  float attenuationDistance;
  float thickness;     /* thinGlass */
  b200_texture baseColorMap; /* principled map_baseColor (rgb x baseColor, alpha x opacity); obj map_kd (rgb x
                                kd, alpha x d); looked up at the hit's texture coordinates; null: none */
  float specular;        /* principled, default 1 */
  float ior;             /* principled, default 1 */
  float diffuse;         /* principled, default 1 */
  float edgeColor[3];    /* principled, default 1 */
  int specularMetallic;  /* principled, default 1: the conductor's weight x specular */
} b200_material;
/* the reference's defaults for a material of `type` (principled: baseColor
 * 0.8, roughness 0, metallic 0, opacity 1; obj: kd 0.8, ks 0, ns 10, d 1,
 * tf 0; metal: aluminium, roughness 0.1; glass: etaInside 1.5, etaOutside
 * 1, attenuation colour 1 over distance 1; thinGlass: eta 1.5, attenuation
 * colour 1, distance 1, thickness 1) */
void b200_material_defaults(b200_material *m, int type);
typedef struct {
  int pixelSamples;        /* spp */
  int maxPathLength;       /* default 20 */
  int roulettePathLength;  /* default 5 */
  int maxScatteringEvents; /* default 20 */
  int lightSamples;        /* default -1: all lights at the first bounce */
  int limitIndirectLightSamples; /* default 1 */
  float minContribution;   /* default 0.001 */
  float maxContribution;   /* default inf */
  float backgroundColor[4];
  int pixelFilter;
  int collectStats;
  b200_texture backplate; /* "map_backplate" (Renderer_getBackground render/Renderer.ispc:19-29): looked up at
                             the pixel centre for paths that see the background straight; null: the
                             background colour */
  float mipMapBias;       /* "mipMapBias" (Renderer.cpp:41): footprint x 2^bias for MIP level selection */
  b200_texture maxDepth;  /* "map_maxDepth" (Renderer_getMaxDepth render/Renderer.ispc:30-40, PathTracer.ispc:
                             189-192): the camera ray's tfar = max(0, texel.r) at the sample's screen position */
} b200_pt_params;
int b200_render_pt(b200_scene scene, const b200_camera_desc *camera, const b200_pt_params *params,
                   const b200_material *materials, int nmaterials, b200_frame fb, void *stream);

/* ---- path tracer for callers that cannot allocate device memory.
 * No counterpart in the reference: OSPRay's CPU device allocates freely.
 * For applications that reserve all device memory up front, must not stall
 * on the allocator inside a real-time loop, or run under an external memory
 * cap, this renders exactly like b200_render_pt but takes its scratch (path
 * workspace, material list, microfacet albedo tables) from a fixed 48 MiB
 * static device array inside the library instead of cudaMalloc; the call
 * itself allocates nothing.  Limits: width * height * pixelSamples <=
 * 190,000 paths and nmaterials <= 4096, else B200_INVALID_ARGUMENT with a
 * message.  The first call on a device sets the scratch up (looks up its
 * device address and fills the albedo tables) and waits for that; make it
 * before capturing any stream.  Calls share the one array: two calls that
 * overlap on the GPU race and must not be issued. */
int b200_render_pt_noalloc(b200_scene scene, const b200_camera_desc *camera, const b200_pt_params *params,
                           const b200_material *materials, int nmaterials, b200_frame fb, void *stream);

/* ---- structured-regular volume + piecewise-linear transfer function
 *      (StructuredRegular volume, volume/Volume.cpp:60-222;
 *       VolumetricModel::commit volume/VolumetricModel.cpp:30-82;
 *       LinearTransferFunction::commit volume/transferFunction/LinearTransferFunction.cpp:22-155).
 * data: nx*ny*nz float, x fastest; vertex-centred grid at origin + i*spacing.
 * color: ncolor x 3 float, opacity: nopacity float over valueRange.
 * One volumetric model per world; a second call replaces it. */
int b200_scene_set_volume(b200_scene scene, const float *data, int nx, int ny, int nz, const float *origin,
                          const float *spacing, const float *color, int ncolor, const float *opacity, int nopacity,
                          const float *valueRange, float densityScale);

/* Gradient shading of the volume (VolumetricModel::commit
 * volume/VolumetricModel.cpp:76 "gradientShadingScale", used by
 * integrateVolumeIntervalsGradient render/scivis/volumes.ispc:384-414):
 * 0 (the default) renders the transfer function's colour; s > 0 shades each sample of non-zero opacity like a surface (Blinn-Phong over the
 * lights, shadows and AO as the SciVis parameters ask) with normal
 * -normalize(gradient) and blends the shaded RGBA into it by s.  The gradient
 * is the finite difference of the trilinear sample at one grid spacing
 * (forward; backward at the upper boundary).  Values <= 0 turn it off; a
 * non-finite value is refused.  Kept across b200_scene_set_volume calls. */
int b200_scene_set_volume_gradient_shading(b200_scene scene, float gradientShadingScale);

/* The volume's instance transform (Instance "transform" of the instance
 * whose group holds the volumetric model; rays go to volume space by its
 * inverse, transformRay render/scivis/volumes.ispc:311-313, and gradient
 * normals back by the inverse transpose): xfm 3x4 row-major as
 * b200_scene_add_instance takes it, null = identity.  Kept across
 * b200_scene_set_volume calls; a singular transform is refused. */
int b200_scene_set_volume_transform(b200_scene scene, const float *xfm);

/* ---- SciVis renderer (SciVis::commit render/scivis/SciVis.cpp:27-84,
 *      SciVis_renderSample render/scivis/SciVis.ispc:24-222,
 *      SciVis_computeShading render/scivis/surfaces.ispc:90-128,
 *      lightAlpha render/scivis/lightAlpha.ispc:19-122).
 * Worlds with surfaces: Blinn-Phong over the non-ambient lights of
 * b200_scene_set_lights (area lights sampled at their centre), hard shadows
 * through translucent surfaces and the volume when `shadows` is set, AO
 * (`aoSamples` rays up to `aoDistance`) tinted by the summed ambient
 * radiance x pi, lights seen directly when `visibleLights` is set, and the
 * volume (if any) composited in front of each surface.  Volume-only worlds
 * take a dedicated kernel unless the volume is gradient shaded
 * (b200_scene_set_volume_gradient_shading). */
typedef struct {
  int pixelSamples;
  float volumeSamplingRate; /* default 1 */
  float backgroundColor[4];
  int pixelFilter;
  int collectStats;         /* volume-only worlds: [rays, volume samples, 0, 0]; else traversal counters */
  int shadows;              /* default 0 */
  int visibleLights;        /* default 0 */
  int aoSamples;            /* default 0 */
  float aoDistance;         /* default 1e20 */
  float minContribution;    /* default 0.001 */
  b200_texture backplate;   /* "map_backplate" at the pixel centre (null: backgroundColor) */
  b200_texture maxDepth;    /* "map_maxDepth" at the pixel centre (null: no depth limit) */
  float mipMapBias;         /* footprint x 2^bias for map_kd level selection */
} b200_scivis_params;
/* The material parameters SciVis reads (evalMaterial,
 * render/scivis/surfaces.ih:44-84): isObj != 0 for an "obj" material (kd,
 * ks, ns, d, tf as in OBJMaterial::commit render/materials/OBJ.cpp); any
 * other material shades white and opaque.  material_id of an instance
 * indexes this array; ids outside it shade with the defaults. */
typedef struct b200_scivis_material_t {
  int isObj;
  float kd[3], ks[3];
  float ns, d;
  float tf[3];
  b200_texture kdMap; /* obj "map_kd": kd x texel rgb, d x texel alpha (surfaces.ih:66-72); null: none */
} b200_scivis_material;
int b200_render_scivis(b200_scene scene, const b200_camera_desc *camera, const b200_scivis_params *params,
                       const b200_scivis_material *materials, int nmaterials, b200_frame fb, void *stream);

/* Traversal counters accumulated by renders with collectStats set:
 * [rays traced, BVH node visits, triangle tests, sphere tests]; reset != 0
 * zeroes them after reading.  (Frame statistics; the reference reports only
 * task durations, ospGetTaskDuration.) */
int b200_scene_counters(b200_scene scene, int64_t *out4, int reset);
int b200_render_ao(b200_scene scene, const b200_camera_desc *camera, const b200_ao_params *params, b200_frame fb,
                   void *stream);

/* ---- batched rendering: many render requests served by one wavefront.
 * No counterpart in the reference, which renders one frame per
 * ospRenderFrame call (ISPCDevice::renderFrame, modules/cpu/ISPCDevice.cpp:
 * 578-595).  A batch holds requests, each a (scene, camera, renderer
 * parameters, framebuffer) as b200_render_ao / b200_render_pt take them;
 * b200_batch_render renders one frame of every request: the paths of all
 * requests share one set of wavefront queues (each ray traverses its own
 * request's scene), in waves of whole pixels, and each framebuffer
 * accumulates exactly as the single-request call would (AO: bit-identical;
 * path tracer: up to the order of the shadow-ray additions).  The frame runs
 * as wavefront kernels (directly or as a replayed CUDA graph) or as one
 * persistent launch (b200_batch_render's mode).  Scenes and
 * framebuffers must outlive the batch; parameters and materials are copied
 * at the add call.  AO requests trace up to two AO rays per sample through
 * the shadow queue and further ones in place. */
typedef struct b200_batch_t *b200_batch;
int b200_batch_create(b200_device dev, b200_batch *out);
int b200_batch_release(b200_batch batch);
int b200_batch_add_ao(b200_batch batch, b200_scene scene, const b200_camera_desc *camera,
                      const b200_ao_params *params, b200_frame fb);
int b200_batch_add_pt(b200_batch batch, b200_scene scene, const b200_camera_desc *camera,
                      const b200_pt_params *params, const b200_material *materials, int nmaterials, b200_frame fb);
/* launch shape: path slots per wave (the workspace, 264 bytes per slot) and
 * resident blocks per SM of the persistent trace and shade kernels (the
 * persistent mode runs every co-resident block and uses wavePaths only) */
typedef struct {
  int64_t wavePaths;
  int traceBlocksPerSM;
  int shadeBlocksPerSM;
} b200_batch_tuning;
int b200_batch_get_tuning(b200_batch batch, b200_batch_tuning *out);
int b200_batch_set_tuning(b200_batch batch, const b200_batch_tuning *tuning);
/* The autotuner: renders the batch once per candidate launch shape (wave
 * sizes x trace / shade residency; wave sizes only when the last render
 * used B200_BATCH_PERSISTENT), timed with CUDA events after one warm-up
 * render, and keeps the fastest; `candidates` <= 0 tries the full set.  The
 * framebuffers are reset afterwards (their accumulation restarts).  The
 * chosen shape is returned in `best` (may be null). */
int b200_batch_autotune(b200_batch batch, int candidates, b200_batch_tuning *best);
/* How b200_batch_render runs the frame:
 * B200_BATCH_KERNELS     the wavefront kernels of every wave (generate, per
 *                        bounce closest trace / shade / shadow trace,
 *                        finalize) and the post-processing, launched directly;
 * B200_BATCH_GRAPH       the same launches captured once as a CUDA graph and
 *                        replayed;
 * B200_BATCH_PERSISTENT  ONE cooperative persistent launch (captured as a
 *                        one-kernel graph): all co-resident blocks run every
 *                        wave's stages in order, separated by grid-wide
 *                        barriers, pulling queue work dynamically, and
 *                        post-process and stamp the requests each wave
 *                        completes.  A barrier wait is bounded (4 s by default,
 *                        b200_batch_set_barrier_timeout); one that
 *                        runs out makes every block leave the kernel, and the
 *                        next b200_batch_render or b200_batch_timings call
 *                        returns B200_UNKNOWN_ERROR.
 * The results are the same in all three modes (AO bit-identical, path
 * tracing to the order of the shadow-ray additions). */
enum { B200_BATCH_KERNELS = 0, B200_BATCH_GRAPH = 1, B200_BATCH_PERSISTENT = 2 };
/* renders one frame of every request on the device stream in `mode` (a
 * graph is captured on first use and after any change to the requests, the
 * tuning, the mode or a framebuffer's post-processing); other values are
 * refused (B200_INVALID_ARGUMENT) */
int b200_batch_render(b200_batch batch, int mode);
/* the bound of the persistent launch's barrier waits in ns (0: the default
 * of 4 s); a bound shorter than a stage makes the frame fail as a timed-out
 * wait does, which is how the failure path is tested */
int b200_batch_set_barrier_timeout(b200_batch batch, uint64_t ns);
/* after a render has finished (b200_device_sync): each request's completion
 * time in ms after the render began (out n doubles, request order), and the
 * rays the render traced */
int b200_batch_timings(b200_batch batch, double *ms, int n, uint64_t *rays);
/* the plan of the last render: [waves, kernel launches per render, path
 * slots over all requests, requests] */
int b200_batch_info(b200_batch batch, int64_t *info4);

/* ---- neural radiance cache (no counterpart in the reference).
 * A multiresolution hash-grid encoding (16 levels x 2 FP16 features, 2^19
 * entries per level, resolutions 16..2048 over the cube around the bounds)
 * of the position, real spherical harmonics (degree 3, 16 terms) of the
 * direction, the normal, roughness and albedo, into a 64-wide MLP with 4
 * hidden ReLU layers and a 3-wide output, BF16 weights on the 5th-generation
 * tensor cores (tcgen05.mma, 128 samples per tile, FP32 accumulators in
 * tensor memory)
 * with FP32 accumulation; trained with Adam on the relative L2 loss.
 * Records are 16 floats: position[3], direction[3] (unit, pointing away from
 * the surface), normal[3], roughness, albedo[3], target rgb[3] (training) or
 * unused.  Device pointers. */
typedef struct b200_nrc_t *b200_nrc;
typedef struct {
  float boundsLo[3], boundsHi[3];
  float learningRate; /* Adam, default 1e-2 */
  uint32_t seed;      /* parameter initialisation */
} b200_nrc_desc;
int b200_nrc_create(b200_device dev, const b200_nrc_desc *desc, b200_nrc *out);
int b200_nrc_release(b200_nrc nrc);
/* out: n x 3 float radiance */
int b200_nrc_infer(b200_nrc nrc, const float *queries, int64_t n, float *out, void *stream);
/* one Adam step on the mean loss of n samples; loss (device float, may be null) */
int b200_nrc_train(b200_nrc nrc, const float *samples, int64_t n, float *loss, void *stream);
/* the gradients of the mean loss of n samples without a step: weights
 * (17,408 floats: 4 hidden layers 64x64 then the output layer 64x16, each
 * row-major [in][out]) and table (16 x 2^19 x 2 floats), device pointers,
 * each may be null */
int b200_nrc_gradients(b200_nrc nrc, const float *samples, int64_t n, float *wgrad, float *tgrad, float *loss,
                       void *stream);
/* FP32 master parameters in the layouts above (host pointers, may be null) */
int b200_nrc_get_params(b200_nrc nrc, float *weights, float *table);
int b200_nrc_set_params(b200_nrc nrc, const float *weights, const float *table);
/* the grid: lo xyz and 1/extent; per level the scale (N_l - 1) and the dense
 * side length (0 = hashed) */
int b200_nrc_grid(b200_nrc nrc, float *lo_invext4, float *scales16, uint32_t *dense16);

/* Check of the radiance cache's tensor-core building block (no counterpart in
 * the reference): one 128 x n x 64 BF16 product D = A B^T on the device's
 * 5th-generation tensor cores (tcgen05.mma, FP32 accumulator in tensor
 * memory).  Host arrays: a 128 x 64, b n x 64 (rounded to BF16), out 128 x n;
 * n = 16, 32 or 64.  Synchronous. */
int b200_tensor_core_check(b200_device dev, const float *a, const float *b, int n, float *out);

/* ---- path tracing with the radiance cache.  Renders one frame like
 * b200_render_pt, except: every other path, at its first vertex after a
 * diffuse bounce (a bounce off a non-metallic or rough surface), takes the
 * cache's radiance there instead of continuing; `trainPaths` evenly spaced
 * paths per frame (a different subset each frame) are traced in full and
 * their vertices' path-suffix radiance becomes training data; then the
 * cache takes `trainSteps` Adam steps of `trainBatch` samples (when
 * `train`).  The plain path tracer (b200_render_pt) is the same method
 * without the cache. */
typedef struct {
  int trainPaths; /* default 16384 */
  int trainSteps; /* default 4 */
  int trainBatch; /* default 16384 (4 x 16384 = 65,536 samples per frame) */
  int train;      /* default 1 */
  int useCache;   /* default 1; 0: a warm-up frame (plain path tracing that only trains) */
  int epochs;     /* default 1: passes of the trainSteps batches over the frame's samples */
} b200_nrc_frame;
void b200_nrc_frame_defaults(b200_nrc_frame *f);
int b200_render_pt_nrc(b200_scene scene, const b200_camera_desc *camera, const b200_pt_params *params,
                       const b200_material *materials, int nmaterials, b200_frame fb, b200_nrc nrc,
                       const b200_nrc_frame *frame_params, void *stream);

/* ---- pick (ospPick, ospray/include/ospray/ospray.h:338-352; Renderer::pick
 *      render/Renderer.cpp:94-140, Renderer_pick render/Renderer.ispc:43-95).
 * One camera ray through normalised screen position (x, y) in [0,1]^2
 * (origin bottom-left, lens centre, time 0.5), traced closest-hit.  On a hit
 * the world position org + t*dir and the instance / geometric-model /
 * primitive IDs of the instance that was hit; otherwise hasHit 0 and IDs
 * 0xffffffff.  Synchronous. */
typedef struct {
  int hasHit;
  float worldPosition[3];
  uint32_t instID, geomID, primID;
} b200_pick_result;
int b200_pick(b200_scene scene, const b200_camera_desc *camera, float screen_x, float screen_y,
              b200_pick_result *result);

#ifdef __cplusplus
}
#endif

#endif /* B200_H */
