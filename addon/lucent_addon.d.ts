/**
 * Types of the Node-API addon (addon/lucent_napi.c) over the GB300 C ABI
 * (include/lucent.h). The shapes follow the reference's own modules:
 * BVH and BVHOptions (src/math/bvh.ts:18-31), BVHHit (bvh.ts:255-260),
 * PackedScene (src/scene/scene.ts:106-134), RenderSettings and RenderStats
 * (src/renderer.ts:42-96).
 */

/** A native object (device BVH, renderer or batch); freed by dispose() or by the GC. */
export type NativeHandle = { readonly __lucentHandle: unique symbol };

export interface NativeBVHResult {
  nodes: Float32Array;       // 8 floats per node: min.xyz, leftFirst, max.xyz, count (bvh.ts:6-16)
  nodeCount: number;
  triIndices: Uint32Array;
  min: [number, number, number];
  max: [number, number, number];
}

export interface NativeBVHOptions {
  maxLeafSize?: number;      // default 4 (bvh.ts:33)
  bins?: number;             // default 12, at most 32
}

export interface NativeHit {
  t: number;
  triIndex: number;
  u: number;
  v: number;
}

export interface NativeRayHits {
  prim: Int32Array;          // source triangle index, -1 on a miss
  t: Float32Array;           // +Infinity on a miss
  u: Float32Array;
  v: Float32Array;
}

/** packScene's inputs before the BVH-order gather (scene.ts:162-305). */
export interface NativePackedScene {
  positions: Float32Array;   // 9 per triangle, mergeMeshes order
  normals: Float32Array;     // 9 per triangle
  uvs?: Float32Array;        // 6 per triangle
  triMaterial: Int32Array;
  triLight: Int32Array;      // -1 = not a light
  triAlpha: Uint8Array;      // needsAlphaTest (material.ts:111)
  materials: Float32Array;   // packMaterials: 40 floats each (material.ts:121-149)
  spheres?: Float32Array;    // centre + radius, at most 64
  sphereMaterials?: Int32Array;
  sphereLights?: Int32Array;
  lights?: Float32Array;     // 16 floats each (scene.ts:88-95), at most 8
  groundMaterial: number;
  nodes?: Float32Array;      // an optional prebuilt BVH over the same triangles (packScene's `prebuilt`)
  nodeCount?: number;
  triIndices?: Uint32Array;
}

/** uploadLighting's uniforms (renderer.ts:355-413). */
export interface NativeLighting {
  sunEnabled: boolean | number;
  sunDir: [number, number, number];
  sunRadiance: [number, number, number];
  sunCosAngle: number;
  sunPdf: number;
  envWidth: number;
  envHeight: number;
  envRgb: Float32Array;      // RGB, rows top to bottom
  envRotationCos: number;
  envRotationSin: number;
  envIntensity: number;
  envBackground: boolean | number;
  backdrop: [number, number, number];
}

/** uploadCamera's uniforms (renderer.ts:424-439), basis normalised. */
export interface NativeCamera {
  position: [number, number, number];
  right: [number, number, number];
  up: [number, number, number];
  forward: [number, number, number];
  tanHalfFov: number;
  aperture: number;
  focusDistance: number;
}

export interface NativeSettings {
  maxBounces: number;        // RenderSettings.maxBounces
  fireflyClamp: number;      // RenderSettings.fireflyClamp
  temporal: boolean | number;
}

export interface NativeStats {
  samples: number;
  width: number;
  height: number;
  triangles: number;
  bvhNodes: number;
  closestRays: number;
  shadowRays: number;
  traceMs: number;
}

export interface NativeTargets {
  color: Float32Array;       // RGB mean + mean luminance^2, rows bottom to top
  albedo: Float32Array;
  normal: Float32Array;
  history: Float32Array;
}

export interface NativeEnvSampler {
  gridWidth: number;
  gridHeight: number;
  table: Float32Array;       // 4 floats per cell: keep probability, alias, pdfUV, alias pdfUV
  total: number;
}

export interface LucentAddon {
  buildBVH(positions: Float32Array, options?: NativeBVHOptions): NativeBVHResult;
  buildBVHAsync(positions: Float32Array, options?: NativeBVHOptions): Promise<NativeBVHResult>;
  createBVH(nodes: Float32Array, nodeCount: number, triIndices: Uint32Array, positions: Float32Array): NativeHandle;
  intersectBVH(bvh: NativeHandle, origin: ArrayLike<number>, dir: ArrayLike<number>, tMin?: number,
               tMax?: number): NativeHit | null;
  intersectRays(bvh: NativeHandle, rays: Float32Array, tMin?: number, tMax?: number): NativeRayHits;
  createRenderer(width: number, height: number): NativeHandle;
  loadScene(r: NativeHandle, scene: NativePackedScene): void;
  uploadLighting(r: NativeHandle, lighting: NativeLighting): void;
  uploadGround(r: NativeHandle, enabled: boolean, height: number): void;
  uploadCamera(r: NativeHandle, camera: NativeCamera): void;
  applySettings(r: NativeHandle, settings: NativeSettings): void;
  reset(r: NativeHandle): void;
  resize(r: NativeHandle, width: number, height: number): void;
  /** wait = false: return once the samples are queued (read, display and stats wait for them). */
  trace(r: NativeHandle, samples: number, wait?: boolean): void;
  /** Successive waves alternate between two path buffers on the renderer's own streams (default on). */
  setPipelining(r: NativeHandle, on: boolean): void;
  denoise(r: NativeHandle, levels: number, sigmaL?: number, sigmaN?: number, sigmaP?: number): void;
  /** viewWidth/viewHeight: show the image in a canvas of that size (Catmull-Rom preview upsampling). */
  display(r: NativeHandle, denoiseWeight: number, tonemap: 0 | 1 | 2, exposure: number, viewWidth?: number,
          viewHeight?: number): Uint8Array;
  stats(r: NativeHandle): NativeStats;
  read(r: NativeHandle): NativeTargets;
  setMaterials(r: NativeHandle, materials: Float32Array): void;
  backward(r: NativeHandle, samples: number, seed: number, dLdImage: Float32Array, materialCount: number,
           envTexels: number): { dParams: Float32Array; dEnv: Float32Array };
  envSampler(rgb: Float32Array, width: number, height: number, maxWidth?: number): NativeEnvSampler;
  createBatch(renderers: NativeHandle[]): NativeHandle;
  traceBatch(batch: NativeHandle, samples: number): void;
  dispose(handle: NativeHandle): void;
}

declare const addon: LucentAddon;
export default addon;
