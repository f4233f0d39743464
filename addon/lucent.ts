/**
 * TypeScript side of the GB300 binding, written to sit in the reference's tree
 * as src/native/lucent.ts (imports are relative to that place). It keeps the
 * reference's signatures and swaps their bodies for the addon's calls:
 *
 *   buildBVH(positions, options)            src/math/bvh.ts:52
 *   buildBVHAsync(positions)                src/math/bvh-async.ts:8
 *   intersectBVH(bvh, positions, ray, ...)  src/math/bvh.ts:265
 *   NativeRenderer                          the Renderer's scene / camera /
 *                                           settings / render / stats calls
 *                                           (src/renderer.ts:279-864) without
 *                                           its WebGL plumbing
 *
 * The addon (lucent_addon.node) is built from addon/lucent_napi.c against
 * include/lucent.h and liblucent_gpu.so; its types are in
 * addon/lucent_addon.d.ts.
 */
import { AABB } from '../math/aabb';
import type { BVH, BVHHit, BVHOptions } from '../math/bvh';
import type { Ray } from '../math/ray';
import type { Camera } from '../scene/scene';
import type { RenderSettings } from '../renderer';
import native, {
  type NativeBVHResult,
  type NativeHandle,
  type NativeLighting,
  type NativePackedScene,
} from './lucent_addon';

function toBVH(r: NativeBVHResult): BVH {
  return { nodes: r.nodes, nodeCount: r.nodeCount, triIndices: r.triIndices, bounds: new AABB(r.min, r.max) };
}

/** buildBVH (bvh.ts:52): same nodes, triIndices and bounds, built on the GPU. */
export function buildBVH(positions: Float32Array, options: BVHOptions = {}): BVH {
  if (!Number.isInteger(positions.length / 9)) {
    throw new Error(`positions length ${positions.length} is not a multiple of 9`);
  }
  return toBVH(native.buildBVH(positions, options));
}

/** buildBVHAsync (bvh-async.ts:8): the build runs off the JS thread. */
export async function buildBVHAsync(positions: Float32Array): Promise<BVH> {
  return toBVH(await native.buildBVHAsync(positions));
}

/** Device copies of the BVHs intersectBVH has seen, keyed by the BVH object. */
const deviceBVH = new WeakMap<BVH, NativeHandle>();

/** intersectBVH (bvh.ts:265): the same hit, decided in binary64 on the GPU. */
export function intersectBVH(bvh: BVH, positions: Float32Array, ray: Ray, tMin = 1e-5, tMax = Infinity): BVHHit | null {
  let h = deviceBVH.get(bvh);
  if (!h) {
    h = native.createBVH(bvh.nodes, bvh.nodeCount, bvh.triIndices, positions);
    deviceBVH.set(bvh, h);
  }
  return native.intersectBVH(h, ray.origin, ray.dir, tMin, tMax);
}

const TONEMAPS = { aces: 0, reinhard: 1, none: 2 } as const;

/**
 * The Renderer's GPU work (renderer.ts:171-871) on the GB300 path. The
 * caller keeps the reference's scene preparation (packScene, uploadLighting's
 * uniforms, the camera basis) and hands the results over.
 */
export class NativeRenderer {
  private handle: NativeHandle;
  private materialCount = 0;

  constructor(public width: number, public height: number) {
    this.handle = native.createRenderer(width, height);
  }

  /** loadScene(scene, bvh?) (renderer.ts:279) with packScene's arrays before its
   *  BVH-order gather (scene.ts:162-305); the gather runs on the GPU. */
  loadScene(packed: NativePackedScene, bvh?: BVH): void {
    const desc: NativePackedScene = bvh
      ? { ...packed, nodes: bvh.nodes, nodeCount: bvh.nodeCount, triIndices: bvh.triIndices }
      : packed;
    native.loadScene(this.handle, desc);
    this.materialCount = packed.materials.length / 40;
  }

  uploadLighting(lighting: NativeLighting): void {
    native.uploadLighting(this.handle, lighting);
  }

  uploadGround(enabled: boolean, height: number): void {
    native.uploadGround(this.handle, enabled, height);
  }

  /** uploadCamera (renderer.ts:424): the basis the reference derives from the Camera. */
  uploadCamera(cam: Camera, basis: { right: number[]; up: number[]; forward: number[] }): void {
    native.uploadCamera(this.handle, {
      position: [cam.position[0], cam.position[1], cam.position[2]],
      right: basis.right as [number, number, number],
      up: basis.up as [number, number, number],
      forward: basis.forward as [number, number, number],
      tanHalfFov: Math.tan((cam.fov * Math.PI) / 360),
      aperture: cam.aperture,
      focusDistance: cam.focusDistance,
    });
  }

  applySettings(s: RenderSettings): void {
    native.applySettings(this.handle, { maxBounces: s.maxBounces, fireflyClamp: s.fireflyClamp, temporal: 1 });
  }

  reset(): void {
    native.reset(this.handle);
  }

  resize(width: number, height: number): void {
    this.width = width;
    this.height = height;
    native.resize(this.handle, width, height);
  }

  /** traceSamples (renderer.ts:702): with wait = false the call returns once the samples are queued,
   *  so a frame loop's next trace starts beside this one's last bounces; render, stats and the
   *  read-back wait for them. */
  trace(samples: number, wait = true): void {
    native.trace(this.handle, samples, wait);
  }

  /** Pipelined waves (default on; images identical either way). */
  setPipelining(on: boolean): void {
    native.setPipelining(this.handle, on);
  }

  /** render() (renderer.ts:552): accumulate, denoise, display into an RGBA8 canvas. */
  render(samples: number, denoiseLevels: number, denoiseWeight: number, tonemap: keyof typeof TONEMAPS,
         exposure: number): Uint8Array {
    native.trace(this.handle, samples);
    if (denoiseLevels > 0) native.denoise(this.handle, denoiseLevels);
    return native.display(this.handle, denoiseLevels > 0 ? denoiseWeight : 0, TONEMAPS[tonemap], exposure);
  }

  stats() {
    return native.stats(this.handle);
  }

  /** Differentiable rendering (no reference counterpart): forward and backward of one image. */
  setMaterials(materials: Float32Array): void {
    native.setMaterials(this.handle, materials);
  }

  backward(samples: number, seed: number, dLdImage: Float32Array, envTexels = 0) {
    return native.backward(this.handle, samples, seed, dLdImage, this.materialCount, envTexels);
  }

  dispose(): void {
    native.dispose(this.handle);
  }
}
