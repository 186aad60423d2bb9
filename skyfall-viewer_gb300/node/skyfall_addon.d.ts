// Types of the N-API addon in skyfall_addon.c (the C-ABI of include/skyfall.h
// as Node sees it).  Every function throws an Error whose `code` is the
// SKY_ERR_* name of a failing status and whose message is sky_last_error().

export type Context = { readonly __skyfallContext: unique symbol };

export interface AddonCamera {
  view: Float32Array;   // 16, column-major world -> camera
  proj: Float32Array;   // 16, column-major projection
  focal: Float32Array;  // fx, fy in pixels
  width: number;
  height: number;
}

export interface StepStats {
  iteration: number;
  loss: number;          // sum over pixels/channels of 0.5 w_l2 r^2 + w_l1 |r|
  intersections: number;
  gaussians: number;
  views: number;
  shDegree: number;
  shUpdated: number;
}

export interface AddonConfig {
  lr_means?: number; lr_sh?: number; lr_opacity?: number; lr_scale?: number; lr_rotation?: number;
  sh_update_interval?: number;
  w_l2?: number; w_l1?: number; w_ssim?: number;
  fwdBatch?: number; bwdBatch?: number; tileCull?: number;
  /** 1: a step of B views scales the learning rates by sqrt(B) and the betas to the power B */
  batchScaling?: number;
}

export interface CreateOptions extends AddonConfig {
  tileSize?: number; shDegree?: number; shDegreeInterval?: number; useGraph?: number;
  maxViewsPerStep?: number; backwardMode?: number; seed?: number;
}

export interface AddonStatus {
  iteration: number; adamSteps: number; lastIntersections: number; deviceBytes: number;
  numGaussians: number; numCameras: number; errorFlags: number; kernelLaunches: number;
  graphReplays: number; sceneExtent: number; densifyRuns: number; pruneRuns: number;
}

export interface DensifyOptions {
  gradThreshold?: number; gradAbsThreshold?: number; sizeThreshold?: number;
  minVisibility?: number; importanceThreshold?: number; maxNewRatio?: number; pixelWidth?: number;
}

export interface ScheduleOptions extends DensifyOptions {
  densifyFrom?: number; densifyUntil?: number; densifyInterval?: number;
  pruneFrom?: number; pruneUntil?: number; pruneInterval?: number;
  opacityResetInterval?: number; opacityResetValue?: number; minOpacity?: number;
  maxScreenSize?: number; maxScaleRatio?: number; maxScaleAbsolute?: number; sceneExtent?: number;
}

export interface Addon {
  create(options?: CreateOptions): Context;
  destroy(ctx: Context): void;
  getConfig(ctx: Context): Required<AddonConfig> & { tileSize: number; shDegree: number };
  setConfig(ctx: Context, partial: AddonConfig): void;
  loadPoints(ctx: Context, params: Float32Array, n: number): void;
  loadPacked(ctx: Context, gaussians: Uint32Array, sh: Uint32Array | null, n: number): void;
  loadPly(ctx: Context, path: string): { count: number; shDegree: number };
  savePly(ctx: Context, path: string, shDegree?: number): void;
  saveCheckpoint(ctx: Context, path: string): void;
  loadCheckpoint(ctx: Context, path: string): void;
  knnInit(ctx: Context, sceneExtent?: number): Float32Array;
  setCameras(ctx: Context, cameras: AddonCamera[]): void;
  setTarget(ctx: Context, camera: number, rgb: Float32Array, width: number, height: number): void;
  step(ctx: Context, cameras: Uint32Array): Promise<StepStats>;
  train(ctx: Context, iterations: number, viewsPerStep?: number): Promise<StepStats>;
  render(ctx: Context, cameras: Uint32Array): { rgba: Float32Array; alpha: Float32Array };
  forward(ctx: Context, cameras: Uint32Array): number;
  backward(ctx: Context): Float32Array;
  prune(ctx: Context, params?: { minOpacity?: number; maxScale?: number; maxRemoveRatio?: number },
        mask?: Uint8Array | null): number;
  resetOpacity(ctx: Context, maxOpacity?: number): void;
  scoreViews(ctx: Context, cameras: Uint32Array | null): { importance: Uint32Array; pruning: Float32Array };
  densify(ctx: Context, options?: DensifyOptions): { cloned: number; split: number };
  pruneScored(ctx: Context, options?: {
    minOpacity?: number; maxScale?: number; maxScreenRadius?: number; useScreenSizePruning?: number;
    pruneRatio?: number; maxRatio?: number; useLastScores?: number }): number;
  setSchedule(ctx: Context, options?: ScheduleOptions | boolean): void;
  getStatus(ctx: Context): AddonStatus;
  getParams(ctx: Context): Float32Array;
  setProfiling(ctx: Context, level: 0 | 1 | 2): void;
  getStageTimes(ctx: Context): { steps: number; ms: Float64Array };
  frame(ctx: Context, camera: AddonCamera, settings?: { gaussianScaling?: number; shDegree?: number }): Uint8Array;
}

declare const addon: Addon;
export default addon;
