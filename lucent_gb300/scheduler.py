"""GPU-budget scheduling over the C ABI, mirroring the reference's
src/perf.ts and Renderer.traceBudgeted (src/renderer.ts:618-649).

A progressive path tracer would keep a GPU at 100% forever; the reference
schedules its work against a budget, the share of wall-clock time the GPU may
spend rendering. GpuBudget is its token bucket (perf.ts:90-115),
affordable_samples the per-frame sample count (perf.ts:118-122), recommend the
preset chosen from a measured scan (perf.ts:65-84). BudgetedRenderer drives a
Renderer with them, taking the cost of a sample from the renderer's own device
timing (lucent_render_stats.last_trace_ms, the counterpart of the reference's
timer queries, renderer.ts:668-700).
"""
import math
import time
from dataclasses import asdict, dataclass, replace

from .renderer import Renderer


@dataclass(frozen=True)
class PerformanceSettings:
    """perf.ts:10-22."""
    gpu_budget: float
    fps_cap: int
    resolution_scale: float
    max_bounces: int
    max_samples: int
    pause_when_unfocused: bool


PERFORMANCE_PRESETS = {  # perf.ts:24-29
    "eco": PerformanceSettings(0.25, 30, 0.5, 4, 1024, True),
    "balanced": PerformanceSettings(0.5, 60, 0.75, 6, 2048, True),
    "high": PerformanceSettings(0.8, 60, 1.0, 8, 4096, True),
    "max": PerformanceSettings(1.0, 0, 1.0, 12, 0, False),
}
PRESET_ORDER = ("eco", "balanced", "high", "max")


def pick_performance(settings):
    """pickPerformance (perf.ts:41-44): the performance fields of a larger settings object."""
    return PerformanceSettings(**{k: getattr(settings, k) for k in PerformanceSettings.__dataclass_fields__})


def match_preset(s):
    """matchPreset (perf.ts:47-50): the preset these settings equal, else 'custom'."""
    for name in PRESET_ORDER:
        if asdict(PERFORMANCE_PRESETS[name]) == asdict(s):
            return name
    return "custom"


@dataclass
class Recommendation:
    preset: str
    settings: PerformanceSettings
    ms_at_1080p: float


def recommend(ms_per_sample, width, height):
    """recommend (perf.ts:65-84): the tier from the cost of a 1080p sample, then
    the resolution lowered in quarter steps (never below 0.25, never above
    the tier's own) until one sample fits the tier's frame-time target."""
    pixels = max(1, width * height)
    ms1080 = ms_per_sample * (1920 * 1080) / pixels
    preset = "high" if ms1080 <= 30 else "balanced" if ms1080 <= 90 else "eco"
    target = 20 if preset == "high" else 25 if preset == "balanced" else 33
    base = PERFORMANCE_PRESETS[preset]
    fit = math.sqrt(target / max(ms_per_sample, 1e-3))
    scale = min(base.resolution_scale, max(0.25, math.floor(fit * 4) / 4))
    return Recommendation(preset, replace(base, resolution_scale=scale), ms1080)


class GpuBudget:
    """Token bucket for GPU time (perf.ts:90-115): wall-clock time earns
    `budget` ms of GPU work per ms; work spends it; savings are capped at
    `burst_ms` and a gap longer than 250 ms is not banked."""

    def __init__(self, budget):
        self.budget = budget
        self.credit = 0.0
        self.last = -1.0

    def allowance(self, now, burst_ms):
        dt = 0.0 if self.last < 0 else min(now - self.last, 250.0)
        self.last = now
        self.credit = min(self.credit + dt * self.budget, max(burst_ms, 1.0))
        return self.credit

    def spend(self, ms):
        self.credit -= ms

    def reset(self):
        self.credit = 0.0
        self.last = -1.0


def render_size(width, height, resolution_scale):
    """Internal resolution (renderer.ts:479-480): the display size scaled and
    rounded half up, at least one pixel."""
    return (max(1, int(math.floor(width * resolution_scale + 0.5))),
            max(1, int(math.floor(height * resolution_scale + 0.5))))


def affordable_samples(allowance_ms, ms_per_sample, cap=32):
    """affordableSamples (perf.ts:118-122): whole samples the allowance pays for."""
    if not (ms_per_sample > 0) or allowance_ms < ms_per_sample:
        return 0
    return min(cap, int(math.floor(allowance_ms / ms_per_sample)))


class BudgetedRenderer:
    """traceBudgeted (renderer.ts:618-649) over a Renderer: each frame() spends
    the frame's share of the GPU budget on samples. The cost of a sample is an
    exponential average of the renderer's measured device time per sample
    (0.8 / 0.2 like pollTimers, renderer.ts:692); the first frame measures one
    sample. `interactive` frames (camera moving) always get one sample;
    `samples_per_frame` > 0 bypasses the budget with a fixed count."""

    def __init__(self, renderer: Renderer, settings: PerformanceSettings, clock=time.perf_counter,
                 samples_per_frame=0):
        self.r = renderer
        self.settings = settings
        self.samples_per_frame = samples_per_frame
        self.budget = GpuBudget(settings.gpu_budget)
        self.ms_per_sample = 0.0
        self.clock = clock
        self.busy_ms = 0.0

    def apply(self, display_width, display_height):
        """Applies the settings' bounce limit and internal resolution to the
        renderer (which restarts its accumulation)."""
        self.r.settings.max_bounces = self.settings.max_bounces
        self.r.apply_settings()
        w, h = render_size(display_width, display_height, self.settings.resolution_scale)
        if (w, h) != (self.r.width, self.r.height):
            self.r.resize(w, h)

    def _now(self):
        return self.clock() * 1e3

    def _trace(self, n):
        self.r.trace_samples(n)
        self.r.check()
        ms = self.r.stats()["last_trace_ms"]
        self.busy_ms += ms
        per = ms / n
        self.ms_per_sample = per if self.ms_per_sample <= 0 else self.ms_per_sample * 0.8 + per * 0.2
        return ms

    def frame(self, interactive=False):
        """One frame's work; returns the samples traced."""
        s = self.settings
        remaining = s.max_samples - self.r.samples() if s.max_samples > 0 else math.inf
        if remaining <= 0:
            return 0
        if self.samples_per_frame > 0:
            n = int(min(self.samples_per_frame, remaining))
            self._trace(n)
            return n
        now = self._now()
        self.budget.budget = s.gpu_budget
        frame_ms = 1000.0 / (s.fps_cap if s.fps_cap > 0 else 60)
        if self.ms_per_sample <= 0:  # measureSample (renderer.ts:652-658)
            self.budget.allowance(now, 0)
            self.budget.spend(self._trace(1))
            return 1
        allowance = self.budget.allowance(now, max(frame_ms * s.gpu_budget * 2, self.ms_per_sample * 1.05))
        n = min(1 if interactive else affordable_samples(allowance, self.ms_per_sample), remaining)
        if n <= 0:
            return 0
        self.budget.spend(n * self.ms_per_sample)
        self._trace(int(n))
        return int(n)
