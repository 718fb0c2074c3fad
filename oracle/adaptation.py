"""ORACLE (test infrastructure only): the thermalisation's step-size adaptation of the
reference, restated to replay the engine's driver cycle by cycle.

Simulation::evaluateMoleculeMoveCounter / evaluateScalingMoveCounter
(core/Simulation.cpp:533-607): a sampler is evaluated once 100 x N of its moves (N requested
moves per cycle) have been made since its last evaluation, the box scaler after 100 box
moves; above 20 % acceptance the step grows by 1.1 (TranslationSampler.cpp:48-54: refused at
the implicit maximum, half the smallest box height; RotationSampler.cpp:36-44: capped at pi;
TriclinicBoxScaler.cpp:9-12), below 10 % it shrinks by 1.1.
"""
from __future__ import annotations

import math


class Counter:
    def __init__(self):
        self.since = 0
        self.since_accepted = 0

    def add(self, moves: int, accepted: int):
        self.since += moves
        self.since_accepted += accepted

    def rate(self) -> float:
        return self.since_accepted / self.since

    def reset(self):
        self.since = self.since_accepted = 0


class Adaptation:
    def __init__(self, n: int, translation_step: float, rotation_step: float, box_step: float,
                 rototranslation: bool = False):
        self.n = n
        self.t, self.r, self.b = translation_step, rotation_step, box_step
        self.ct, self.cr, self.cb = Counter(), Counter(), Counter()
        self.rototranslation = rototranslation

    def evaluate(self, max_translation: float):
        if self.rototranslation:
            # RototranslationSampler::increaseStepSize / decreaseStepSize
            # (core/move_samplers/RototranslationSampler.cpp:50-61, :87-93); its moves are
            # counted with the rotations
            if self.cr.since >= 100 * self.n:
                rate = self.cr.rate()
                self.cr.reset()
                if rate > 0.2:
                    old = self.t
                    if not (max_translation > 0 and self.t >= max_translation):
                        self.t *= 1.1
                    self.r *= self.t / old
                elif rate < 0.1:
                    self.t /= 1.1
                    self.r /= 1.1
            self._box()
            return
        if self.t > 0 and self.ct.since >= 100 * self.n:
            rate = self.ct.rate()
            self.ct.reset()
            if rate > 0.2:
                if not (max_translation > 0 and self.t >= max_translation):
                    self.t *= 1.1
            elif rate < 0.1:
                self.t /= 1.1
        if self.r > 0 and self.cr.since >= 100 * self.n:
            rate = self.cr.rate()
            self.cr.reset()
            if rate > 0.2:
                self.r *= 1.1
                if self.r > math.pi:
                    self.r = math.pi
            elif rate < 0.1:
                self.r /= 1.1
        self._box()

    def _box(self):
        if self.b > 0 and self.cb.since >= 100:
            rate = self.cb.rate()
            self.cb.reset()
            if rate > 0.2:
                self.b *= 1.1
            elif rate < 0.1:
                self.b /= 1.1
