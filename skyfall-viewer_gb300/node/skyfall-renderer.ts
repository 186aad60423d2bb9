// SkyfallRenderer -- the TypeScript host of Skyfall-Viewer's render-and-train
// hot path on libskyfall (CUDA, GB300) through the N-API addon in
// skyfall_addon.c.
//
// It keeps the method names, argument meaning and return types of the
// GaussianRenderer interface (src/renderers/gaussian-renderer.ts:30-58) for
// the training path, so src/renderers/renderer.ts can hold either object,
// and adds the forward/backward op pair.  Differences that follow from the
// host:
//  * cameras are TrainingCameraData as in the reference, but training
//    images are CPU pixel arrays (Float32 RGB, row-major, y down) instead of
//    GPU textures -- setTrainingImages takes {data, width, height};
//  * frame() returns RGBA8 pixels (to put into a canvas) instead of drawing
//    into a WebGPU texture, and KNN initialisation needs no encoder;
//  * camera choice in train() comes from the library's seeded generator.
// Calls on one context are serialised through a promise queue: the addon's
// step()/train() run on a worker and a context takes one call at a time.

import addon, { type AddonCamera, type Context, type StepStats } from './skyfall_addon';

export interface TrainingCameraData {
  view: Float32Array;      // world -> camera, column-major
  proj: Float32Array;      // projection, column-major
  focal: Float32Array | [number, number];
  imgSize: Float32Array | [number, number];  // (w, h)
}

export interface TrainingImage {
  data: Float32Array;      // width * height * 3, RGB in [0, 1]
  width: number;
  height: number;
}

// gaussian-renderer.ts:99-122, training-controller.ts:49-54
export interface TrainingParams {
  lr_means: number; lr_sh: number; lr_opacity: number; lr_scale: number; lr_rotation: number;
  sh_update_interval: number;
}
export interface LossWeights { w_l2: number; w_l1: number; w_ssim: number; }
export interface TrainingStatus {
  isTraining: boolean; currentIteration: number; targetIterations: number;
  iterationsPerSecond: number; gaussianCount: number;
}
export interface PruneParams {
  minOpacity: number; maxScale: number; maxScreenRadius: number; useScreenSizePruning: boolean;
}

const STAGES = ['preprocess', 'scan', 'emit', 'sort', 'ranges', 'forward', 'backward', 'geom_adam'];

function toAddonCamera(c: TrainingCameraData): AddonCamera {
  return {
    view: Float32Array.from(c.view), proj: Float32Array.from(c.proj),
    focal: Float32Array.from(c.focal), width: c.imgSize[0], height: c.imgSize[1],
  };
}

export class SkyfallRenderer {
  private readonly ctx: Context;
  private queue: Promise<unknown> = Promise.resolve();
  private cameras: TrainingCameraData[] = [];
  private viewport: [number, number] = [0, 0];
  private gaussianScale = 1.0;
  private isTraining = false;
  private stopRequested = false;
  private targetIterations = 0;
  private startTime = 0;
  private completed = 0;
  private viewsPerStep = 1;

  constructor(options: { tileSize?: number; shDegree?: number; useGraph?: boolean;
                         maxViewsPerStep?: number; seed?: number } = {}) {
    this.ctx = addon.create({
      tileSize: options.tileSize, shDegree: options.shDegree ?? 3,
      useGraph: options.useGraph === false ? 0 : 1,
      maxViewsPerStep: options.maxViewsPerStep ?? 16, seed: options.seed,
    });
  }

  // one call at a time on the context
  private serial<T>(fn: () => T | Promise<T>): Promise<T> {
    const run = this.queue.then(fn, fn);
    this.queue = run.catch(() => undefined);
    return run;
  }

  // ---- scene ----------------------------------------------------------------
  /** reloadPointCloud: 59 planes of n floats (position, log sigma,
   *  quaternion x y z w, opacity logit, 48 SH) */
  loadPoints(params: Float32Array, n: number): void { addon.loadPoints(this.ctx, params, n); }
  /** the reference's packed f16 buffers as they are (common.wgsl:39-43) */
  loadPacked(gaussians: Uint32Array, sh: Uint32Array | null, n: number): void {
    addon.loadPacked(this.ctx, gaussians, sh, n);
  }
  /** loadPlyFile + reloadPointCloud */
  loadPly(path: string): { count: number; shDegree: number } { return addon.loadPly(this.ctx, path); }
  savePly(path: string, shDegree = 3): void { addon.savePly(this.ctx, path, shDegree); }
  saveCheckpoint(path: string): void { addon.saveCheckpoint(this.ctx, path); }
  loadCheckpoint(path: string): void { addon.loadCheckpoint(this.ctx, path); }
  async initializeKnnAndSync(): Promise<void> {
    await this.serial(() => { addon.knnInit(this.ctx, 0); });
  }
  initializeKnn(): void { addon.knnInit(this.ctx, 0); }
  getSceneExtent(): number { return addon.getStatus(this.ctx).sceneExtent; }

  setTrainingCameras(cameras: TrainingCameraData[]): void {
    this.cameras = cameras;
    addon.setCameras(this.ctx, cameras.map(toAddonCamera));
  }
  setTrainingImages(images: TrainingImage[]): void {
    if (this.cameras.length > 0 && images.length !== this.cameras.length)
      console.warn(`Image count (${images.length}) doesn't match camera count (${this.cameras.length}).`);
    images.forEach((im, i) => addon.setTarget(this.ctx, i, im.data, im.width, im.height));
  }
  /** intersections are built on the device by every pass: nothing to do */
  async buildTrainingTiles(): Promise<void> { /* per pass, on the device */ }

  // ---- training (train :3744-3854, trainStep :3638-3660) ---------------------
  /** numFrames steps of viewsPerStep seeded cameras each (1 = the reference) */
  async train(numFrames: number, viewsPerStep = this.viewsPerStep): Promise<void> {
    if (this.isTraining || numFrames <= 0) return;
    this.isTraining = true;
    this.stopRequested = false;
    this.targetIterations = numFrames;
    this.startTime = performance.now();
    this.completed = 0;
    try {
      for (let i = 0; i < numFrames && !this.stopRequested; i++) {
        await this.serial(() => addon.train(this.ctx, 1, viewsPerStep));
        this.completed++;
      }
    } finally {
      this.isTraining = false;
      this.stopRequested = false;
    }
  }
  stopTraining(): void { if (this.isTraining) this.stopRequested = true; }
  /** one training step over the given cameras (batched: one launch per stage) */
  step(cameras: number[]): Promise<StepStats> {
    return this.serial(() => addon.step(this.ctx, Uint32Array.from(cameras)));
  }
  setViewsPerStep(views: number): void { this.viewsPerStep = Math.max(1, Math.min(64, views)); }
  async profiledTrainStep(): Promise<void> {
    await this.serial(() => addon.train(this.ctx, 1, this.viewsPerStep));
  }

  // ---- the forward / backward op pair ----------------------------------------
  /** renders the cameras and evaluates the loss against their targets */
  forward(cameras: number[]): Promise<number> {
    return this.serial(() => addon.forward(this.ctx, Uint32Array.from(cameras)));
  }
  /** gradients of the last forward's loss: 59 planes of n floats, no Adam step */
  backward(): Promise<Float32Array> { return this.serial(() => addon.backward(this.ctx)); }
  /** rendered training views, RGBA f32 and alpha, concatenated */
  render(cameras: number[]): Promise<{ rgba: Float32Array; alpha: Float32Array }> {
    return this.serial(() => addon.render(this.ctx, Uint32Array.from(cameras)));
  }

  // ---- prune / densify / opacity reset ---------------------------------------
  /** prune(customParams?) (:2177-2212): the multi-view weighted prune; returns
   *  the Gaussian count after it */
  async prune(customParams?: PruneParams): Promise<number> {
    await this.serial(() => addon.pruneScored(this.ctx, customParams ? {
      minOpacity: customParams.minOpacity, maxScale: customParams.maxScale,
      maxScreenRadius: customParams.maxScreenRadius,
      useScreenSizePruning: customParams.useScreenSizePruning ? 1 : 0,
    } : undefined));
    return this.getGaussianCount();
  }
  /** rule or mask prune without the random budget */
  async pruneByRule(minOpacity = 0.005, maxScale = Infinity, mask?: Uint8Array): Promise<number> {
    return this.serial(() => addon.prune(this.ctx, { minOpacity, maxScale: Math.min(maxScale, 3.4e38) },
                                         mask ?? null));
  }
  async densify(): Promise<{ cloned: number; split: number }> {
    return this.serial(() => addon.densify(this.ctx));
  }
  async resetOpacity(maxOpacity = 0.1): Promise<void> {
    await this.serial(() => addon.resetOpacity(this.ctx, maxOpacity));
  }
  /** TrainingController schedule run by train(); false disables it */
  setSchedule(options: Parameters<typeof addon.setSchedule>[1] = {}): void {
    addon.setSchedule(this.ctx, options);
  }

  // ---- parameters, loss weights, status --------------------------------------
  getTrainingParams(): TrainingParams {
    const c = addon.getConfig(this.ctx);
    return { lr_means: c.lr_means, lr_sh: c.lr_sh, lr_opacity: c.lr_opacity, lr_scale: c.lr_scale,
             lr_rotation: c.lr_rotation, sh_update_interval: c.sh_update_interval };
  }
  setTrainingParams(params: Partial<TrainingParams>): void { addon.setConfig(this.ctx, params); }
  getLossWeights(): LossWeights {
    const c = addon.getConfig(this.ctx);
    return { w_l2: c.w_l2, w_l1: c.w_l1, w_ssim: c.w_ssim };
  }
  setLossWeights(weights: Partial<LossWeights>): void { addon.setConfig(this.ctx, weights); }
  getTrainingStatus(): TrainingStatus {
    const st = addon.getStatus(this.ctx);
    const elapsed = this.isTraining ? (performance.now() - this.startTime) / 1000 : 0;
    return { isTraining: this.isTraining, currentIteration: st.iteration,
             targetIterations: this.targetIterations,
             iterationsPerSecond: elapsed > 0 ? this.completed / elapsed : 0,
             gaussianCount: st.numGaussians };
  }
  getGaussianCount(): number { return addon.getStatus(this.ctx).numGaussians; }
  /** splat-batch depths and culled lists: speed only, results unchanged */
  setBatchDepth(fwdBatch = 0, bwdBatch = 0): void { addon.setConfig(this.ctx, { fwdBatch, bwdBatch }); }
  setTileCull(on = true): void { addon.setConfig(this.ctx, { tileCull: on ? 1 : 0 }); }
  /** Adam hyperparameters of multi-view steps: lr x sqrt(B), betas^B (one-view steps unchanged) */
  setBatchScaling(on = true): void { addon.setConfig(this.ctx, { batchScaling: on ? 1 : 0 }); }

  // ---- profiling (TrainingProfiler) ------------------------------------------
  enableProfiling(enabled: boolean): void { addon.setProfiling(this.ctx, enabled ? 1 : 0); }
  printProfilingReport(): void {
    const t = addon.getStageTimes(this.ctx);
    const steps = Math.max(1, t.steps);
    console.log(`[profiler] ${t.steps} steps`);
    STAGES.forEach((name, k) => console.log(`  ${name.padEnd(12)} ${(t.ms[k] / steps).toFixed(3)} ms`));
  }
  async dumpTrainingDiagnostics(): Promise<void> {
    const st = addon.getStatus(this.ctx);
    console.log('[diagnostics]', JSON.stringify(st));
  }

  // ---- viewer ------------------------------------------------------------------
  setGaussianScale(value: number): void { this.gaussianScale = value; }
  resizeViewport(w: number, h: number): void { this.viewport = [w, h]; }
  /** frame(encoder, view) of the viewer, headless: RGBA8 pixels of the camera,
   *  to put into a canvas (ImageData) or upload into a texture */
  frame(camera: { view: Float32Array; proj: Float32Array; focal: [number, number] },
        shDegree = 3): Uint8Array {
    const [w, h] = this.viewport;
    return addon.frame(this.ctx, { view: camera.view, proj: camera.proj,
                                   focal: Float32Array.from(camera.focal), width: w, height: h },
                       { gaussianScaling: this.gaussianScale, shDegree });
  }

  destroy(): void { addon.destroy(this.ctx); }
}

export default function get_renderer(options?: ConstructorParameters<typeof SkyfallRenderer>[0]) {
  return new SkyfallRenderer(options);
}
