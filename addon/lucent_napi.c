/*
 * Node-API binding of the GB300 hot path (include/lucent.h) for the
 * reference's TypeScript host. The TypeScript modules keep their signatures
 * (src/math/bvh.ts:52, 265; src/math/bvh-async.ts:8; src/renderer.ts:171-871)
 * and call this addon instead of their CPU loops and WebGL passes; see
 * addon/lucent.ts for that wrapper and addon/lucent_addon.d.ts for the types.
 *
 * Conventions:
 *  - typed arrays are read in place (no copy) and results come back as new
 *    typed arrays the addon allocates;
 *  - a failing call throws a JS Error carrying lucent_last_error(), as the
 *    reference throws Error (bvh.ts:55-57, scene.ts:163-165, ...);
 *  - handles (BVH, renderer, batch) are JS externals whose finalizers free the
 *    native object; dispose() frees it early, as Renderer.dispose does
 *    (renderer.ts:864-870);
 *  - buildBVHAsync runs the build on a libuv worker (napi_create_async_work),
 *    the counterpart of the reference's Web Worker (bvh-async.ts:12-30).
 *
 * Build (a maintainer's node-gyp target): sources addon/lucent_napi.c, include
 * dir include/, link lucent_gb300/_build/liblucent_gpu.so.
 */
#include <node_api.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>

#include "../include/lucent.h"

/* ------------------------------------------------------------------ helpers */
#define CHECK_NAPI(env, call)                                  \
  do {                                                         \
    if ((call) != napi_ok) {                                   \
      napi_throw_error((env), NULL, "N-API call failed: " #call); \
      return NULL;                                             \
    }                                                          \
  } while (0)

static napi_value throw_last(napi_env env) {
  const char* msg = lucent_last_error();
  napi_throw_error(env, NULL, msg && msg[0] ? msg : "lucent call failed");
  return NULL;
}

static napi_value undefined(napi_env env) {
  napi_value u;
  napi_get_undefined(env, &u);
  return u;
}

/* Data pointer and element count of a typed array of the given type. */
static int typed_array(napi_env env, napi_value v, napi_typedarray_type want, void** data, size_t* len) {
  bool is = false;
  if (napi_is_typedarray(env, v, &is) != napi_ok || !is) return 0;
  napi_typedarray_type type;
  napi_value ab;
  size_t off;
  if (napi_get_typedarray_info(env, v, &type, len, data, &ab, &off) != napi_ok || type != want) return 0;
  return 1;
}

/* New typed array of n elements; *data receives its storage. */
static napi_value new_typed(napi_env env, napi_typedarray_type type, size_t elem, size_t n, void** data) {
  napi_value ab, out;
  if (napi_create_arraybuffer(env, elem * (n ? n : 1), data, &ab) != napi_ok) return NULL;
  if (napi_create_typedarray(env, type, n, ab, 0, &out) != napi_ok) return NULL;
  return out;
}

static int get_double(napi_env env, napi_value obj, const char* key, double* out) {
  bool has = false;
  napi_value v;
  if (napi_has_named_property(env, obj, key, &has) != napi_ok || !has) return 0;
  if (napi_get_named_property(env, obj, key, &v) != napi_ok) return 0;
  return napi_get_value_double(env, v, out) == napi_ok;
}

static float prop_f(napi_env env, napi_value obj, const char* key, float dflt) {
  double d;
  return get_double(env, obj, key, &d) ? (float)d : dflt;
}

static void prop_vec3(napi_env env, napi_value obj, const char* key, float out[3]) {
  napi_value v, e;
  bool has = false;
  if (napi_has_named_property(env, obj, key, &has) != napi_ok || !has) return;
  if (napi_get_named_property(env, obj, key, &v) != napi_ok) return;
  for (uint32_t i = 0; i < 3; i++) {
    double d;
    if (napi_get_element(env, v, i, &e) == napi_ok && napi_get_value_double(env, e, &d) == napi_ok) out[i] = (float)d;
  }
}

static void* prop_typed(napi_env env, napi_value obj, const char* key, napi_typedarray_type type, size_t* len) {
  napi_value v;
  bool has = false;
  void* data = NULL;
  *len = 0;
  if (napi_has_named_property(env, obj, key, &has) != napi_ok || !has) return NULL;
  if (napi_get_named_property(env, obj, key, &v) != napi_ok) return NULL;
  if (!typed_array(env, v, type, &data, len)) return NULL;
  return data;
}

static napi_value set_num(napi_env env, napi_value obj, const char* key, double x) {
  napi_value v;
  napi_create_double(env, x, &v);
  napi_set_named_property(env, obj, key, v);
  return obj;
}

static napi_value vec3(napi_env env, const double* x) {
  napi_value arr, v;
  napi_create_array_with_length(env, 3, &arr);
  for (uint32_t i = 0; i < 3; i++) {
    napi_create_double(env, x[i], &v);
    napi_set_element(env, arr, i, v);
  }
  return arr;
}

/* External handles: the finalizer frees the native object unless dispose ran. */
typedef struct handle {
  int kind; /* 1 BVH, 2 renderer, 3 batch */
  void* ptr;
} handle;

static void finalize_handle(napi_env env, void* data, void* hint) {
  (void)env;
  (void)hint;
  handle* h = (handle*)data;
  if (h->ptr) {
    if (h->kind == 1) lucent_bvh_destroy((lucent_bvh*)h->ptr);
    if (h->kind == 2) lucent_renderer_destroy((lucent_renderer*)h->ptr);
    if (h->kind == 3) lucent_batch_destroy((lucent_batch*)h->ptr);
  }
  free(h);
}

static napi_value wrap(napi_env env, int kind, void* ptr) {
  handle* h = (handle*)malloc(sizeof(handle));
  napi_value out;
  if (!h) return NULL;
  h->kind = kind;
  h->ptr = ptr;
  if (napi_create_external(env, h, finalize_handle, NULL, &out) != napi_ok) {
    free(h);
    return NULL;
  }
  return out;
}

static handle* unwrap(napi_env env, napi_value v, int kind) {
  void* data = NULL;
  if (napi_get_value_external(env, v, &data) != napi_ok || !data) return NULL;
  handle* h = (handle*)data;
  return h->kind == kind && h->ptr ? h : NULL;
}

static napi_value args(napi_env env, napi_callback_info info, size_t want, napi_value* argv, size_t* argc) {
  *argc = want;
  if (napi_get_cb_info(env, info, argc, argv, NULL, NULL) != napi_ok) return NULL;
  return argv[0];
}

/* ------------------------------------------------------------------ BVH */
/* {nodes, nodeCount, triIndices, min, max} from a finished build. */
static napi_value bvh_result(napi_env env, const float* nodes, uint32_t count, const uint32_t* tri, uint32_t n_tri,
                             const double* bounds) {
  void *nd, *td;
  napi_value out, nodes_v = new_typed(env, napi_float32_array, 4, (size_t)count * 8, &nd);
  napi_value tri_v = new_typed(env, napi_uint32_array, 4, n_tri, &td);
  if (!nodes_v || !tri_v) return NULL;
  memcpy(nd, nodes, (size_t)count * 8 * sizeof(float));
  if (n_tri) memcpy(td, tri, (size_t)n_tri * sizeof(uint32_t));
  napi_create_object(env, &out);
  napi_set_named_property(env, out, "nodes", nodes_v);
  set_num(env, out, "nodeCount", count);
  napi_set_named_property(env, out, "triIndices", tri_v);
  napi_set_named_property(env, out, "min", vec3(env, bounds));
  napi_set_named_property(env, out, "max", vec3(env, bounds + 3));
  return out;
}

static void read_opts(napi_env env, napi_value obj, lucent_bvh_opts* o) {
  double d;
  o->max_leaf_size = 4;
  o->bins = 12;
  if (!obj) return;
  if (get_double(env, obj, "maxLeafSize", &d)) o->max_leaf_size = (uint32_t)d;
  if (get_double(env, obj, "bins", &d)) o->bins = (uint32_t)d;
}

/* buildBVH(positions: Float32Array, options?) (bvh.ts:52). */
static napi_value BuildBVH(napi_env env, napi_callback_info info) {
  napi_value argv[2];
  size_t argc;
  args(env, info, 2, argv, &argc);
  void* pos;
  size_t len;
  if (argc < 1 || !typed_array(env, argv[0], napi_float32_array, &pos, &len)) {
    napi_throw_type_error(env, NULL, "positions must be a Float32Array");
    return NULL;
  }
  lucent_bvh_opts o;
  read_opts(env, argc > 1 ? argv[1] : NULL, &o);
  const uint32_t n = (uint32_t)(len / 9);
  float* nodes = (float*)malloc(sizeof(float) * 8 * (n ? 2 * (size_t)n - 1 : 1));
  uint32_t* tri = (uint32_t*)malloc(sizeof(uint32_t) * (n ? n : 1));
  uint32_t count = 0;
  double bounds[6];
  napi_value out = NULL;
  if (!nodes || !tri) {
    napi_throw_error(env, NULL, "out of host memory");
  } else if (lucent_bvh_build((const float*)pos, len, &o, nodes, &count, tri, bounds, NULL, NULL)) {
    throw_last(env);
  } else {
    out = bvh_result(env, nodes, count, tri, n, bounds);
  }
  free(nodes);
  free(tri);
  return out;
}

/* buildBVHAsync(positions) (bvh-async.ts:8): the same build on a worker
 * thread; the positions are copied first, as the reference transfers a copy
 * to its worker (bvh-async.ts:29). */
typedef struct build_job {
  napi_async_work work;
  napi_deferred deferred;
  float* pos;
  uint64_t len;
  lucent_bvh_opts opts;
  float* nodes;
  uint32_t* tri;
  uint32_t count;
  double bounds[6];
  lucent_status status;
  char error[512];
} build_job;

static void build_execute(napi_env env, void* data) {
  (void)env;
  build_job* j = (build_job*)data;
  const uint32_t n = (uint32_t)(j->len / 9);
  j->nodes = (float*)malloc(sizeof(float) * 8 * (n ? 2 * (size_t)n - 1 : 1));
  j->tri = (uint32_t*)malloc(sizeof(uint32_t) * (n ? n : 1));
  if (!j->nodes || !j->tri) {
    j->status = LUCENT_ERR_OOM;
    strcpy(j->error, "out of host memory");
    return;
  }
  j->status = lucent_bvh_build(j->pos, j->len, &j->opts, j->nodes, &j->count, j->tri, j->bounds, NULL, NULL);
  if (j->status) strncpy(j->error, lucent_last_error(), sizeof j->error - 1); /* the worker thread's message */
}

static void build_complete(napi_env env, napi_status status, void* data) {
  build_job* j = (build_job*)data;
  napi_value v = NULL, err, msg;
  if (status == napi_ok && j->status == LUCENT_OK)
    v = bvh_result(env, j->nodes, j->count, j->tri, (uint32_t)(j->len / 9), j->bounds);
  if (v) {
    napi_resolve_deferred(env, j->deferred, v);
  } else {
    napi_create_string_utf8(env, j->status ? j->error : "BVH build failed", NAPI_AUTO_LENGTH, &msg);
    napi_create_error(env, NULL, msg, &err);
    napi_reject_deferred(env, j->deferred, err);
  }
  napi_delete_async_work(env, j->work);
  free(j->pos);
  free(j->nodes);
  free(j->tri);
  free(j);
}

static napi_value BuildBVHAsync(napi_env env, napi_callback_info info) {
  napi_value argv[2], promise, name;
  size_t argc;
  args(env, info, 2, argv, &argc);
  void* pos;
  size_t len;
  if (argc < 1 || !typed_array(env, argv[0], napi_float32_array, &pos, &len)) {
    napi_throw_type_error(env, NULL, "positions must be a Float32Array");
    return NULL;
  }
  build_job* j = (build_job*)calloc(1, sizeof(build_job));
  if (!j || !(j->pos = (float*)malloc(sizeof(float) * (len ? len : 1)))) {
    free(j);
    napi_throw_error(env, NULL, "out of host memory");
    return NULL;
  }
  memcpy(j->pos, pos, sizeof(float) * len);
  j->len = len;
  read_opts(env, argc > 1 ? argv[1] : NULL, &j->opts);
  CHECK_NAPI(env, napi_create_promise(env, &j->deferred, &promise));
  napi_create_string_utf8(env, "lucent.buildBVHAsync", NAPI_AUTO_LENGTH, &name);
  CHECK_NAPI(env, napi_create_async_work(env, NULL, name, build_execute, build_complete, j, &j->work));
  CHECK_NAPI(env, napi_queue_async_work(env, j->work));
  return promise;
}

/* createBVH(nodes, nodeCount, triIndices, positions): the device copy behind
 * intersectBVH's (bvh, positions) pair (bvh.ts:265). */
static napi_value CreateBVH(napi_env env, napi_callback_info info) {
  napi_value argv[4];
  size_t argc;
  args(env, info, 4, argv, &argc);
  void *nodes, *tri, *pos;
  size_t nl, tl, pl;
  uint32_t count = 0;
  if (argc < 4 || !typed_array(env, argv[0], napi_float32_array, &nodes, &nl) ||
      napi_get_value_uint32(env, argv[1], &count) != napi_ok ||
      !typed_array(env, argv[2], napi_uint32_array, &tri, &tl) ||
      !typed_array(env, argv[3], napi_float32_array, &pos, &pl)) {
    napi_throw_type_error(env, NULL, "createBVH(nodes: Float32Array, nodeCount, triIndices: Uint32Array, "
                                     "positions: Float32Array)");
    return NULL;
  }
  if ((size_t)count * 8 > nl || pl != tl * 9) {
    napi_throw_error(env, NULL, "BVH arrays do not match nodeCount / positions");
    return NULL;
  }
  lucent_bvh* b = NULL;
  if (lucent_bvh_create((const float*)nodes, count, (const uint32_t*)tri, (uint32_t)tl, (const float*)pos, &b))
    return throw_last(env);
  return wrap(env, 1, b);
}

/* intersectBVH(handle, origin, dir, tMin = 1e-5, tMax = Infinity) ->
 * {t, triIndex, u, v} | null, in binary64 like the reference's Ray (ray.ts:4-7). */
static napi_value IntersectBVH(napi_env env, napi_callback_info info) {
  napi_value argv[5];
  size_t argc;
  args(env, info, 5, argv, &argc);
  handle* h = argc >= 3 ? unwrap(env, argv[0], 1) : NULL;
  if (!h) {
    napi_throw_type_error(env, NULL, "intersectBVH(bvh, origin, dir, tMin?, tMax?)");
    return NULL;
  }
  double ray[6] = {0, 0, 0, 0, 0, 0}, t_min = 1e-5, t_max = 1.0 / 0.0;
  for (int k = 0; k < 2; k++)
    for (uint32_t i = 0; i < 3; i++) {
      napi_value e;
      if (napi_get_element(env, argv[1 + k], i, &e) == napi_ok) napi_get_value_double(env, e, &ray[3 * k + i]);
    }
  if (argc > 3) napi_get_value_double(env, argv[3], &t_min);
  if (argc > 4) napi_get_value_double(env, argv[4], &t_max);
  int32_t prim = -1;
  double t, u, v;
  if (lucent_bvh_intersect_f64((lucent_bvh*)h->ptr, ray, 1, t_min, t_max, &prim, &t, &u, &v, NULL))
    return throw_last(env);
  if (prim < 0) {
    napi_value nul;
    napi_get_null(env, &nul);
    return nul;
  }
  napi_value out;
  napi_create_object(env, &out);
  set_num(env, out, "t", t);
  set_num(env, out, "triIndex", prim);
  set_num(env, out, "u", u);
  return set_num(env, out, "v", v);
}

/* intersectRays(handle, rays: Float32Array (6 per ray), tMin, tMax) ->
 * {prim: Int32Array, t, u, v: Float32Array}: many rays in one call. */
static napi_value IntersectRays(napi_env env, napi_callback_info info) {
  napi_value argv[4];
  size_t argc;
  args(env, info, 4, argv, &argc);
  handle* h = argc >= 2 ? unwrap(env, argv[0], 1) : NULL;
  void* rays;
  size_t len;
  if (!h || !typed_array(env, argv[1], napi_float32_array, &rays, &len) || len % 6) {
    napi_throw_type_error(env, NULL, "intersectRays(bvh, rays: Float32Array of 6 floats per ray, tMin?, tMax?)");
    return NULL;
  }
  double t_min = 1e-5, t_max = 1.0 / 0.0;
  if (argc > 2) napi_get_value_double(env, argv[2], &t_min);
  if (argc > 3) napi_get_value_double(env, argv[3], &t_max);
  const uint32_t n = (uint32_t)(len / 6);
  void *p, *t, *u, *v;
  napi_value pv = new_typed(env, napi_int32_array, 4, n, &p), tv = new_typed(env, napi_float32_array, 4, n, &t);
  napi_value uv = new_typed(env, napi_float32_array, 4, n, &u), vv = new_typed(env, napi_float32_array, 4, n, &v);
  if (!pv || !tv || !uv || !vv) return NULL;
  if (lucent_bvh_intersect((lucent_bvh*)h->ptr, (const float*)rays, n, t_min, t_max, (int32_t*)p, (float*)t,
                           (float*)u, (float*)v, NULL))
    return throw_last(env);
  napi_value out;
  napi_create_object(env, &out);
  napi_set_named_property(env, out, "prim", pv);
  napi_set_named_property(env, out, "t", tv);
  napi_set_named_property(env, out, "u", uv);
  napi_set_named_property(env, out, "v", vv);
  return out;
}

/* ------------------------------------------------------------------ renderer */
static lucent_renderer* renderer_arg(napi_env env, napi_value v) {
  handle* h = unwrap(env, v, 2);
  if (!h) napi_throw_type_error(env, NULL, "expected a renderer handle");
  return h ? (lucent_renderer*)h->ptr : NULL;
}

/* createRenderer(width, height) (new Renderer(canvas), renderer.ts:226). */
static napi_value CreateRenderer(napi_env env, napi_callback_info info) {
  napi_value argv[2];
  size_t argc;
  args(env, info, 2, argv, &argc);
  uint32_t w = 0, h = 0;
  if (argc < 2 || napi_get_value_uint32(env, argv[0], &w) != napi_ok ||
      napi_get_value_uint32(env, argv[1], &h) != napi_ok) {
    napi_throw_type_error(env, NULL, "createRenderer(width, height)");
    return NULL;
  }
  lucent_renderer* r = NULL;
  if (lucent_renderer_create(w, h, &r)) return throw_last(env);
  return wrap(env, 2, r);
}

/* loadScene(r, packed) (renderer.ts:279): the PackedScene inputs
 * (scene.ts:106-134) before the BVH-order gather, as typed arrays:
 * positions, normals, uvs?, triMaterial, triLight, triAlpha (Uint8Array),
 * materials, spheres?, sphereMaterials?, sphereLights?, lights?, groundMaterial,
 * and optionally a prebuilt BVH (nodes, nodeCount, triIndices). */
static napi_value LoadScene(napi_env env, napi_callback_info info) {
  napi_value argv[2];
  size_t argc;
  args(env, info, 2, argv, &argc);
  lucent_renderer* r = argc >= 2 ? renderer_arg(env, argv[0]) : NULL;
  if (!r) return NULL;
  napi_value o = argv[1];
  lucent_scene_desc d;
  size_t n;
  memset(&d, 0, sizeof d);
  d.positions = (const float*)prop_typed(env, o, "positions", napi_float32_array, &n);
  d.tri_count = (uint32_t)(n / 9);
  d.normals = (const float*)prop_typed(env, o, "normals", napi_float32_array, &n);
  d.uvs = (const float*)prop_typed(env, o, "uvs", napi_float32_array, &n);
  d.tri_material = (const int32_t*)prop_typed(env, o, "triMaterial", napi_int32_array, &n);
  d.tri_light = (const int32_t*)prop_typed(env, o, "triLight", napi_int32_array, &n);
  d.tri_alpha = (const uint8_t*)prop_typed(env, o, "triAlpha", napi_uint8_array, &n);
  d.materials = (const float*)prop_typed(env, o, "materials", napi_float32_array, &n);
  d.material_count = (uint32_t)(n / 40);
  d.spheres = (const float*)prop_typed(env, o, "spheres", napi_float32_array, &n);
  d.sphere_count = (uint32_t)(n / 4);
  d.sphere_materials = (const int32_t*)prop_typed(env, o, "sphereMaterials", napi_int32_array, &n);
  d.sphere_lights = (const int32_t*)prop_typed(env, o, "sphereLights", napi_int32_array, &n);
  d.lights = (const float*)prop_typed(env, o, "lights", napi_float32_array, &n);
  d.light_count = (uint32_t)(n / 16);
  d.ground_material = (int32_t)prop_f(env, o, "groundMaterial", -1.f);
  d.bvh_nodes = (const float*)prop_typed(env, o, "nodes", napi_float32_array, &n);
  d.bvh_node_count = (uint32_t)prop_f(env, o, "nodeCount", 0.f);
  d.bvh_tri_indices = (const uint32_t*)prop_typed(env, o, "triIndices", napi_uint32_array, &n);
  if (lucent_renderer_load_scene(r, &d)) return throw_last(env);
  return undefined(env);
}

/* uploadLighting(r, {sunEnabled, sunDir, sunRadiance, sunCosAngle, sunPdf,
 * envWidth, envHeight, envRgb, envRotationCos, envRotationSin, envIntensity,
 * envBackground, backdrop}) (renderer.ts:355-413); the caller computes the
 * uniforms as uploadLighting does (Math.cos / Math.sin of the rotation). */
static napi_value UploadLighting(napi_env env, napi_callback_info info) {
  napi_value argv[2];
  size_t argc;
  args(env, info, 2, argv, &argc);
  lucent_renderer* r = argc >= 2 ? renderer_arg(env, argv[0]) : NULL;
  if (!r) return NULL;
  napi_value o = argv[1];
  lucent_lighting l;
  size_t n;
  memset(&l, 0, sizeof l);
  l.sun_enabled = prop_f(env, o, "sunEnabled", 0.f) != 0.f;
  prop_vec3(env, o, "sunDir", l.sun_dir);
  prop_vec3(env, o, "sunRadiance", l.sun_radiance);
  l.sun_cos_angle = prop_f(env, o, "sunCosAngle", 1.f);
  l.sun_pdf = prop_f(env, o, "sunPdf", 0.f);
  l.env_width = (uint32_t)prop_f(env, o, "envWidth", 0.f);
  l.env_height = (uint32_t)prop_f(env, o, "envHeight", 0.f);
  l.env_rgb = (const float*)prop_typed(env, o, "envRgb", napi_float32_array, &n);
  if (l.env_rgb && n != (size_t)l.env_width * l.env_height * 3) {
    napi_throw_error(env, NULL, "envRgb must hold envWidth * envHeight * 3 floats");
    return NULL;
  }
  l.env_rotation_cos = prop_f(env, o, "envRotationCos", 1.f);
  l.env_rotation_sin = prop_f(env, o, "envRotationSin", 0.f);
  l.env_intensity = prop_f(env, o, "envIntensity", 1.f);
  l.env_background = prop_f(env, o, "envBackground", 1.f) != 0.f;
  prop_vec3(env, o, "backdrop", l.backdrop);
  if (lucent_renderer_upload_lighting(r, &l)) return throw_last(env);
  return undefined(env);
}

/* uploadGround(r, enabled, height) (renderer.ts:415-421). */
static napi_value UploadGround(napi_env env, napi_callback_info info) {
  napi_value argv[3];
  size_t argc;
  args(env, info, 3, argv, &argc);
  lucent_renderer* r = argc >= 3 ? renderer_arg(env, argv[0]) : NULL;
  if (!r) return NULL;
  bool on = false;
  double hgt = 0;
  napi_get_value_bool(env, argv[1], &on);
  napi_get_value_double(env, argv[2], &hgt);
  if (lucent_renderer_upload_ground(r, on ? 1 : 0, (float)hgt)) return throw_last(env);
  return undefined(env);
}

/* uploadCamera(r, {position, right, up, forward, tanHalfFov, aperture,
 * focusDistance}) (renderer.ts:424-439), basis already normalised. */
static napi_value UploadCamera(napi_env env, napi_callback_info info) {
  napi_value argv[2];
  size_t argc;
  args(env, info, 2, argv, &argc);
  lucent_renderer* r = argc >= 2 ? renderer_arg(env, argv[0]) : NULL;
  if (!r) return NULL;
  lucent_camera c;
  memset(&c, 0, sizeof c);
  prop_vec3(env, argv[1], "position", c.position);
  prop_vec3(env, argv[1], "right", c.right);
  prop_vec3(env, argv[1], "up", c.up);
  prop_vec3(env, argv[1], "forward", c.forward);
  c.tan_half_fov = prop_f(env, argv[1], "tanHalfFov", 0.41421356f);
  c.aperture = prop_f(env, argv[1], "aperture", 0.f);
  c.focus_distance = prop_f(env, argv[1], "focusDistance", 5.f);
  if (lucent_renderer_upload_camera(r, &c)) return throw_last(env);
  return undefined(env);
}

/* applySettings(r, {maxBounces, fireflyClamp, temporal}) (renderer.ts:454-460). */
static napi_value ApplySettings(napi_env env, napi_callback_info info) {
  napi_value argv[2];
  size_t argc;
  args(env, info, 2, argv, &argc);
  lucent_renderer* r = argc >= 2 ? renderer_arg(env, argv[0]) : NULL;
  if (!r) return NULL;
  lucent_settings s;
  s.max_bounces = (uint32_t)prop_f(env, argv[1], "maxBounces", 6.f);
  s.firefly_clamp = prop_f(env, argv[1], "fireflyClamp", 8.f);
  s.temporal = prop_f(env, argv[1], "temporal", 1.f) != 0.f;
  if (lucent_renderer_apply_settings(r, &s)) return throw_last(env);
  return undefined(env);
}

/* reset(r) (renderer.ts:463), dispose(r) (renderer.ts:864). */
static napi_value Reset(napi_env env, napi_callback_info info) {
  napi_value argv[1];
  size_t argc;
  args(env, info, 1, argv, &argc);
  lucent_renderer* r = argc >= 1 ? renderer_arg(env, argv[0]) : NULL;
  if (!r) return NULL;
  if (lucent_renderer_reset(r)) return throw_last(env);
  return undefined(env);
}

static napi_value Dispose(napi_env env, napi_callback_info info) {
  napi_value argv[1];
  size_t argc;
  args(env, info, 1, argv, &argc);
  for (int kind = 1; kind <= 3 && argc >= 1; kind++) {
    handle* h = unwrap(env, argv[0], kind);
    if (!h) continue;
    if (kind == 1) lucent_bvh_destroy((lucent_bvh*)h->ptr);
    if (kind == 2) lucent_renderer_destroy((lucent_renderer*)h->ptr);
    if (kind == 3) lucent_batch_destroy((lucent_batch*)h->ptr);
    h->ptr = NULL;
  }
  return undefined(env);
}

/* resize(r, width, height) (renderer.ts:476). */
static napi_value Resize(napi_env env, napi_callback_info info) {
  napi_value argv[3];
  size_t argc;
  args(env, info, 3, argv, &argc);
  lucent_renderer* r = argc >= 3 ? renderer_arg(env, argv[0]) : NULL;
  if (!r) return NULL;
  uint32_t w = 0, h = 0;
  napi_get_value_uint32(env, argv[1], &w);
  napi_get_value_uint32(env, argv[2], &h);
  if (lucent_renderer_resize(r, w, h)) return throw_last(env);
  return undefined(env);
}

/* trace(r, samples, wait = true): the accumulation half of render()
 * (renderer.ts:552-620, the traceSamples draw loop :702-736). With wait it
 * returns after the samples finished; with wait = false it returns once they
 * are queued, so that the next frame's waves can start beside this frame's
 * last bounces (pipelined waves); read, display and stats wait for them. */
static napi_value Trace(napi_env env, napi_callback_info info) {
  napi_value argv[3];
  size_t argc;
  args(env, info, 3, argv, &argc);
  lucent_renderer* r = argc >= 2 ? renderer_arg(env, argv[0]) : NULL;
  if (!r) return NULL;
  uint32_t samples = 0;
  bool wait = true;
  napi_get_value_uint32(env, argv[1], &samples);
  if (argc >= 3) napi_get_value_bool(env, argv[2], &wait);  /* undefined keeps the default */
  if (lucent_renderer_trace(r, samples, NULL) || (wait && lucent_renderer_check(r, NULL))) return throw_last(env);
  return undefined(env);
}

/* setPipelining(r, on): successive waves on two path buffers and the
 * renderer's own streams (default on; images identical either way). */
static napi_value SetPipelining(napi_env env, napi_callback_info info) {
  napi_value argv[2];
  size_t argc;
  args(env, info, 2, argv, &argc);
  lucent_renderer* r = argc >= 2 ? renderer_arg(env, argv[0]) : NULL;
  if (!r) return NULL;
  bool on = true;
  napi_get_value_bool(env, argv[1], &on);
  if (lucent_renderer_set_pipelining(r, on ? 1 : 0)) return throw_last(env);
  return undefined(env);
}

/* denoise(r, levels, sigmaL, sigmaN, sigmaP) (runDenoiser, renderer.ts:788-830). */
static napi_value Denoise(napi_env env, napi_callback_info info) {
  napi_value argv[5];
  size_t argc;
  args(env, info, 5, argv, &argc);
  lucent_renderer* r = argc >= 2 ? renderer_arg(env, argv[0]) : NULL;
  if (!r) return NULL;
  uint32_t levels = 0;
  double sl = 4, sn = 64, sp = 1.5;
  napi_get_value_uint32(env, argv[1], &levels);
  if (argc > 2) napi_get_value_double(env, argv[2], &sl);
  if (argc > 3) napi_get_value_double(env, argv[3], &sn);
  if (argc > 4) napi_get_value_double(env, argv[4], &sp);
  if (lucent_renderer_denoise(r, levels, (float)sl, (float)sn, (float)sp, NULL)) return throw_last(env);
  return undefined(env);
}

/* display(r, denoiseWeight, tonemap (0 ACES, 1 Reinhard, 2 none), exposure
 * [, viewWidth, viewHeight]) -> Uint8Array RGBA8 canvas (rows bottom to top),
 * renderer.ts:573-591; a view size other than the renderer's shows its image
 * through display.frag's Catmull-Rom upsampling (the preview). */
static napi_value Display(napi_env env, napi_callback_info info) {
  napi_value argv[6];
  size_t argc;
  args(env, info, 6, argv, &argc);
  lucent_renderer* r = argc >= 1 ? renderer_arg(env, argv[0]) : NULL;
  if (!r) return NULL;
  double weight = 0, exposure = 1;
  int32_t tonemap = 0;
  if (argc > 1) napi_get_value_double(env, argv[1], &weight);
  if (argc > 2) napi_get_value_int32(env, argv[2], &tonemap);
  if (argc > 3) napi_get_value_double(env, argv[3], &exposure);
  lucent_render_stats st;
  if (lucent_renderer_stats(r, &st)) return throw_last(env);
  uint32_t vw = st.width, vh = st.height;
  if (argc > 5) {
    napi_get_value_uint32(env, argv[4], &vw);
    napi_get_value_uint32(env, argv[5], &vh);
  }
  void* px;
  napi_value out = new_typed(env, napi_uint8_array, 1, (size_t)vw * vh * 4, &px);
  if (!out) return NULL;
  if (lucent_renderer_display_view(r, vw, vh, (float)weight, tonemap, (float)exposure, (uint8_t*)px, NULL, NULL))
    return throw_last(env);
  return out;
}

/* stats(r) (renderer.ts:832-854) plus ray counters and phase times. */
static napi_value Stats(napi_env env, napi_callback_info info) {
  napi_value argv[1];
  size_t argc;
  args(env, info, 1, argv, &argc);
  lucent_renderer* r = argc >= 1 ? renderer_arg(env, argv[0]) : NULL;
  if (!r) return NULL;
  lucent_render_stats st;
  if (lucent_renderer_stats(r, &st)) return throw_last(env);
  napi_value out;
  napi_create_object(env, &out);
  set_num(env, out, "samples", st.samples);
  set_num(env, out, "width", st.width);
  set_num(env, out, "height", st.height);
  set_num(env, out, "triangles", st.triangles);
  set_num(env, out, "bvhNodes", st.bvh_nodes);
  set_num(env, out, "closestRays", (double)st.closest_rays);
  set_num(env, out, "shadowRays", (double)st.shadow_rays);
  return set_num(env, out, "traceMs", st.last_trace_ms);
}

/* read(r) -> {color, albedo, normal: Float32Array (4 per pixel), history}. */
static napi_value Read(napi_env env, napi_callback_info info) {
  napi_value argv[1];
  size_t argc;
  args(env, info, 1, argv, &argc);
  lucent_renderer* r = argc >= 1 ? renderer_arg(env, argv[0]) : NULL;
  if (!r) return NULL;
  lucent_render_stats st;
  if (lucent_renderer_stats(r, &st)) return throw_last(env);
  const size_t px = (size_t)st.width * st.height;
  void *c, *a, *n, *h;
  napi_value cv = new_typed(env, napi_float32_array, 4, px * 4, &c), av = new_typed(env, napi_float32_array, 4, px * 4, &a);
  napi_value nv = new_typed(env, napi_float32_array, 4, px * 4, &n), hv = new_typed(env, napi_float32_array, 4, px, &h);
  if (!cv || !av || !nv || !hv) return NULL;
  if (lucent_renderer_read(r, (float*)c, (float*)a, (float*)n, (float*)h)) return throw_last(env);
  napi_value out;
  napi_create_object(env, &out);
  napi_set_named_property(env, out, "color", cv);
  napi_set_named_property(env, out, "albedo", av);
  napi_set_named_property(env, out, "normal", nv);
  napi_set_named_property(env, out, "history", hv);
  return out;
}

/* setMaterials(r, materials: Float32Array) and backward(r, samples, seed,
 * dLdImage: Float32Array, materialCount, envTexels) -> {dParams, dEnv}: the
 * differentiable renderer's Function pair (no reference counterpart).
 * dParams holds 6 floats per material (base colour rgb, roughness, metallic,
 * clearcoat), dEnv 3 per environment texel (0 texels: no environment
 * gradient). */
static napi_value SetMaterials(napi_env env, napi_callback_info info) {
  napi_value argv[2];
  size_t argc;
  args(env, info, 2, argv, &argc);
  lucent_renderer* r = argc >= 2 ? renderer_arg(env, argv[0]) : NULL;
  void* m;
  size_t n;
  if (!r) return NULL;
  if (!typed_array(env, argv[1], napi_float32_array, &m, &n) || n % 40) {
    napi_throw_type_error(env, NULL, "materials must be a Float32Array of 40 floats per material");
    return NULL;
  }
  if (lucent_renderer_set_materials(r, (const float*)m, (uint32_t)(n / 40))) return throw_last(env);
  return undefined(env);
}

static napi_value Backward(napi_env env, napi_callback_info info) {
  napi_value argv[6];
  size_t argc;
  args(env, info, 6, argv, &argc);
  lucent_renderer* r = argc >= 6 ? renderer_arg(env, argv[0]) : NULL;
  if (!r) return NULL;
  uint32_t samples = 0, seed = 0, mats = 0, env_texels = 0;
  void* dl;
  size_t n;
  napi_get_value_uint32(env, argv[1], &samples);
  napi_get_value_uint32(env, argv[2], &seed);
  napi_get_value_uint32(env, argv[4], &mats);
  napi_get_value_uint32(env, argv[5], &env_texels);
  lucent_render_stats st;
  if (lucent_renderer_stats(r, &st)) return throw_last(env);
  if (!typed_array(env, argv[3], napi_float32_array, &dl, &n) || n != (size_t)st.width * st.height * 4) {
    napi_throw_type_error(env, NULL, "dLdImage must be a Float32Array of width * height * 4 floats");
    return NULL;
  }
  void *dp, *de;
  napi_value dpv = new_typed(env, napi_float32_array, 4, (size_t)mats * 6, &dp);
  napi_value dev = new_typed(env, napi_float32_array, 4, (size_t)env_texels * 3, &de);
  if (!dpv || !dev) return NULL;
  if (lucent_renderer_backward(r, samples, seed, (const float*)dl, (float*)dp, env_texels ? (float*)de : NULL, NULL))
    return throw_last(env);
  napi_value out;
  napi_create_object(env, &out);
  napi_set_named_property(env, out, "dParams", dpv);
  napi_set_named_property(env, out, "dEnv", dev);
  return out;
}

/* envSampler(rgb, width, height, maxWidth = 1024) -> {gridWidth, gridHeight,
 * table, total}: buildEnvSampler (environment.ts:52-85). */
static napi_value EnvSampler(napi_env env, napi_callback_info info) {
  napi_value argv[4];
  size_t argc;
  args(env, info, 4, argv, &argc);
  void* rgb;
  size_t n;
  uint32_t w = 0, h = 0, max_w = 1024;
  if (argc < 3 || !typed_array(env, argv[0], napi_float32_array, &rgb, &n) ||
      napi_get_value_uint32(env, argv[1], &w) != napi_ok || napi_get_value_uint32(env, argv[2], &h) != napi_ok ||
      n != (size_t)w * h * 3) {
    napi_throw_type_error(env, NULL, "envSampler(rgb: Float32Array, width, height, maxWidth?)");
    return NULL;
  }
  if (argc > 3) napi_get_value_uint32(env, argv[3], &max_w);
  uint32_t gw = 0, gh = 0;
  double total = 0;
  if (lucent_env_sampler((const float*)rgb, w, h, max_w, &gw, &gh, NULL, NULL)) return throw_last(env);
  void* tab;
  napi_value tv = new_typed(env, napi_float32_array, 4, (size_t)gw * gh * 4, &tab);
  if (!tv) return NULL;
  if (lucent_env_sampler((const float*)rgb, w, h, max_w, &gw, &gh, (float*)tab, &total)) return throw_last(env);
  napi_value out;
  napi_create_object(env, &out);
  set_num(env, out, "gridWidth", gw);
  set_num(env, out, "gridHeight", gh);
  napi_set_named_property(env, out, "table", tv);
  return set_num(env, out, "total", total);
}

/* ------------------------------------------------------------------ batches */
/* createBatch([renderers]) and traceBatch(batch, samples): several scenes as
 * one wavefront (no reference counterpart). */
static napi_value CreateBatch(napi_env env, napi_callback_info info) {
  napi_value argv[1];
  size_t argc;
  args(env, info, 1, argv, &argc);
  uint32_t n = 0;
  bool is = false;
  if (argc < 1 || napi_is_array(env, argv[0], &is) != napi_ok || !is ||
      napi_get_array_length(env, argv[0], &n) != napi_ok || n == 0) {
    napi_throw_type_error(env, NULL, "createBatch(renderers: array of renderer handles)");
    return NULL;
  }
  lucent_renderer** rs = (lucent_renderer**)malloc(sizeof(lucent_renderer*) * n);
  if (!rs) return NULL;
  for (uint32_t i = 0; i < n; i++) {
    napi_value e;
    napi_get_element(env, argv[0], i, &e);
    handle* h = unwrap(env, e, 2);
    if (!h) {
      free(rs);
      napi_throw_type_error(env, NULL, "createBatch: element is not a renderer handle");
      return NULL;
    }
    rs[i] = (lucent_renderer*)h->ptr;
  }
  lucent_batch* b = NULL;
  lucent_status st = lucent_batch_create(rs, n, &b);
  free(rs);
  if (st) return throw_last(env);
  return wrap(env, 3, b);
}

static napi_value TraceBatch(napi_env env, napi_callback_info info) {
  napi_value argv[2];
  size_t argc;
  args(env, info, 2, argv, &argc);
  handle* h = argc >= 2 ? unwrap(env, argv[0], 3) : NULL;
  if (!h) {
    napi_throw_type_error(env, NULL, "traceBatch(batch, samples)");
    return NULL;
  }
  uint32_t samples = 0;
  napi_get_value_uint32(env, argv[1], &samples);
  if (lucent_batch_trace((lucent_batch*)h->ptr, samples, NULL) || lucent_batch_check((lucent_batch*)h->ptr, NULL, NULL))
    return throw_last(env);
  return undefined(env);
}

/* ------------------------------------------------------------------ module */
static napi_value Init(napi_env env, napi_value exports) {
  const napi_property_descriptor props[] = {
      {"buildBVH", NULL, BuildBVH, NULL, NULL, NULL, napi_default, NULL},
      {"buildBVHAsync", NULL, BuildBVHAsync, NULL, NULL, NULL, napi_default, NULL},
      {"createBVH", NULL, CreateBVH, NULL, NULL, NULL, napi_default, NULL},
      {"intersectBVH", NULL, IntersectBVH, NULL, NULL, NULL, napi_default, NULL},
      {"intersectRays", NULL, IntersectRays, NULL, NULL, NULL, napi_default, NULL},
      {"createRenderer", NULL, CreateRenderer, NULL, NULL, NULL, napi_default, NULL},
      {"loadScene", NULL, LoadScene, NULL, NULL, NULL, napi_default, NULL},
      {"uploadLighting", NULL, UploadLighting, NULL, NULL, NULL, napi_default, NULL},
      {"uploadGround", NULL, UploadGround, NULL, NULL, NULL, napi_default, NULL},
      {"uploadCamera", NULL, UploadCamera, NULL, NULL, NULL, napi_default, NULL},
      {"applySettings", NULL, ApplySettings, NULL, NULL, NULL, napi_default, NULL},
      {"reset", NULL, Reset, NULL, NULL, NULL, napi_default, NULL},
      {"resize", NULL, Resize, NULL, NULL, NULL, napi_default, NULL},
      {"trace", NULL, Trace, NULL, NULL, NULL, napi_default, NULL},
      {"setPipelining", NULL, SetPipelining, NULL, NULL, NULL, napi_default, NULL},
      {"denoise", NULL, Denoise, NULL, NULL, NULL, napi_default, NULL},
      {"display", NULL, Display, NULL, NULL, NULL, napi_default, NULL},
      {"stats", NULL, Stats, NULL, NULL, NULL, napi_default, NULL},
      {"read", NULL, Read, NULL, NULL, NULL, napi_default, NULL},
      {"setMaterials", NULL, SetMaterials, NULL, NULL, NULL, napi_default, NULL},
      {"backward", NULL, Backward, NULL, NULL, NULL, napi_default, NULL},
      {"envSampler", NULL, EnvSampler, NULL, NULL, NULL, napi_default, NULL},
      {"createBatch", NULL, CreateBatch, NULL, NULL, NULL, napi_default, NULL},
      {"traceBatch", NULL, TraceBatch, NULL, NULL, NULL, napi_default, NULL},
      {"dispose", NULL, Dispose, NULL, NULL, NULL, napi_default, NULL},
  };
  if (napi_define_properties(env, exports, sizeof props / sizeof props[0], props) != napi_ok) return NULL;
  return exports;
}

NAPI_MODULE(NODE_GYP_MODULE_NAME, Init)
