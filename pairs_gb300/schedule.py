"""Learned neighbour-list rebuild schedule, trained on the run's own guard trips.

Policy "learned" of LJEngine.  The exact FP64 displacement guard (a particle moved
more than skin/2 since the last list build, evaluated every step inside the
integration kernel) still decides whether a list is valid.  What the network decides is
when the host rebuilds and synchronises:

* Warm-up: the host reads the guard after every step and rebuilds exactly at each
  trip (policy "guard").  At several points of each rebuild cycle the per-cell
  features are stored; when the cycle's trip step s is seen, each stored sample
  (features at step t) gets the label R = s - t (steps that remained).
* Training: Adam on the stored samples, all on the GPU through the library's own
  forward / soft-minimum / backward / Adam kernels.
* Inference: right after every rebuild the network predicts R for the new cycle;
  the host enqueues steps up to the predicted trip without reading anything back,
  then rebuilds proactively.  At a build the sample's features (of the state just
  binned: velocities in the new order, forces read through the binning's
  permutation), the forward pass, the soft minimum and the copy of the prediction to
  the host run on a side stream beside the list build; the force pass, which
  overwrites the forces, waits for them.  If the guard tripped earlier, every force and
  integration pass after the trip did nothing (pg_particles.guard), so the host
  rewinds to the trip step, rebuilds there and continues: a misprediction costs
  skipped launches, never a wrong force.
"""
import ctypes as C
import math

import numpy as np
import torch

from . import _capi as A


class LearnedSchedule:
    def __init__(self, engine, warmup_cycles=6, samples_per_cycle=4, margin=1.1, temperature=0.05, lr=3e-3,
                 train_steps=300, seed=0, max_samples=64, top_cells=256, online_every=32, online_steps=1,
                 online_recent=16):
        self.e = engine
        lib = A.load()
        self.np = lib.pg_mlp_param_count()
        self.ncells_all = engine.cells.ncells
        self.ncells = min(top_cells, self.ncells_all)       # cells per sample: the fastest ones
        # one Adam step on the 16 newest samples every `online_every` cycles keeps the
        # network following the run (~0.5 ms at 1M atoms; every 128 cycles instead of 32
        # left the first cycles' bias in place: 69 rebuilds in 400 steps against 61)
        self.online_every = online_every
        # online calibration of the network's output: an average of log(observed /
        # predicted) cycle length, added to every prediction, takes out what bias the
        # training has not (the network is first trained on the run's first cycles)
        self.calib_rate = 0.3
        self.bias = 0.0
        self._open_pred = None            # raw log prediction for the open cycle
        self._open_start = None
        self.online_steps = online_steps
        self.online_recent = online_recent
        self.warmup_cycles = warmup_cycles
        self.samples_per_cycle = samples_per_cycle
        # steps run without a guard read up to the prediction x margin; a trip before
        # that point is found at the rebuild and the steps after it are redone.  Margins
        # 0.9-1.3 measured at 1M and 131k atoms: 1.05-1.1 fastest (a step redone costs
        # its launches, a rebuild one step early costs a list build)
        self.margin = margin
        self.temperature = temperature
        self.lr = lr
        self.train_steps = train_steps
        self.max_samples = max_samples
        dev = engine.dev
        g = torch.Generator().manual_seed(seed)
        p = torch.zeros(self.np, dtype=torch.float32)
        # Xavier-style init; the output bias starts at log(10 steps)
        H, IN = 64, 3
        p[0:H * IN] = torch.randn(H * IN, generator=g) * math.sqrt(1.0 / IN)
        p[H * IN + H: H * IN + H + H * H] = torch.randn(H * H, generator=g) * math.sqrt(1.0 / H)
        o3 = H * IN + H + H * H + H
        p[o3:o3 + H] = torch.randn(H, generator=g) * math.sqrt(1.0 / H) * 0.1
        p[-1] = math.log(10.0)
        self.params = p.to(dev)
        self.grads = torch.zeros(self.np, dtype=torch.float32, device=dev)
        self.m1 = torch.zeros_like(self.grads)
        self.m2 = torch.zeros_like(self.grads)
        self.adam_t = 0
        self.out = torch.zeros(self.ncells, dtype=torch.float32, device=dev)
        self.result = torch.zeros(4, dtype=torch.float32, device=dev)
        self.result_host = torch.zeros(4, dtype=torch.float32).pin_memory()
        self._next = None
        self.loss = torch.zeros(1, dtype=torch.float32, device=dev)
        self.feat = torch.zeros((max_samples, self.ncells, 4), dtype=torch.float32, device=dev)
        self.feat_all = torch.zeros((self.ncells_all, 4), dtype=torch.float32, device=dev)
        # the prediction at a build runs on a side stream (after the features event)
        self.side = torch.cuda.Stream(device=dev)
        self.side_h = C.c_void_p(self.side.cuda_stream)
        self.ev_feat = torch.cuda.Event()
        self.ev_pred = torch.cuda.Event()
        self._side_busy = False
        self.labels = []                  # (slot, log R, censored)
        self.pending = []                 # (slot, step) samples of the open cycle
        self.cycles = 0
        self.trained = False
        self.history = []                 # (cycle start, predicted R, observed R or None)
        self.train_log = []

    def _ptr(self, t):
        return C.c_void_p(t.data_ptr())

    # ---------------------------------------------------------------- features / prediction
    def features_into(self, slot, since=None):
        """Per-cell features of the current state.  The sample keeps `ncells` cells:
        the fastest of each of `ncells` slabs of the grid, among them the fastest cell
        of the system (the soft minimum is decided by the fast cells)."""
        e = self.e
        since = e.since_build if since is None else since
        A.call("pg_cell_features", C.byref(e.p), C.byref(e.cells), e.precision, since, e.dt,
               0.5 * e.skin, self._ptr(self.feat_all), e.sh)
        if self.ncells == self.ncells_all:
            self.feat[slot].copy_(self.feat_all)
        else:
            A.call("pg_cell_select", self._ptr(self.feat_all), self.ncells_all, self.ncells, self._ptr(self.feat[slot]),
                   e.sh)

    def _side_done(self):
        """Order the engine's stream after the side stream's last prediction (it
        shares the output buffers) and wait for its copy to the host."""
        if self._side_busy:
            self.e.stream.wait_event(self.ev_pred)
            self.ev_pred.synchronize()
            self._side_busy = False

    def predict_log(self, slot, stream=None):
        """Soft-min prediction for the features in `slot` (device scalar in result[0]),
        on the engine's stream or the given stream handle."""
        e = self.e
        if stream is None:
            self._side_done()
        sh = e.sh if stream is None else stream
        A.call("pg_mlp_forward", self._ptr(self.params), self._ptr(self.feat[slot]), self.ncells,
               self._ptr(self.out), sh)
        A.call("pg_mlp_softmin", self._ptr(self.out), self.ncells, self.temperature, self._ptr(self.result), sh)

    def _slot(self):
        used = {s for s, _, _ in self.labels} | {s for s, _ in self.pending}
        for k in range(self.max_samples):
            if k not in used:
                return k
        # overwrite the oldest labelled sample
        s = self.labels.pop(0)[0]
        return s

    # ---------------------------------------------------------------- cycle bookkeeping
    def record(self, step):
        """Store the features of the current state as a sample of the open cycle."""
        slot = self._slot()
        self.features_into(slot)
        self.pending.append((slot, step))

    def sample_after_bin(self, predict):
        """Features of the state at a list rebuild, as the first sample of the new
        cycle (steps since the build = 0), taken on the side stream right after the
        binning: velocities are in the new order, the forces still in the old one and
        read through the binning's permutation (pg_cell_features_binned), so each
        particle's velocity and force stay together.  With `predict`, also the
        network's prediction, copied to host memory.  Returns the event the engine's
        later work (the force pass, which overwrites the forces) waits for."""
        e = self.e
        slot = self._slot()
        self._side_done()
        self.ev_feat.record(e.stream)
        self.side.wait_event(self.ev_feat)
        perm = A.load().pg_bin_permutation(e.n, e.cells.ncells, e.ws)
        if not perm:
            raise A.PairsError("the binning workspace holds no permutation")
        A.call("pg_cell_features_binned", C.byref(e.p), C.byref(e.cells), C.c_void_p(perm), e.precision, 0, e.dt,
               0.5 * e.skin, self._ptr(self.feat_all), self.side_h)
        if self.ncells == self.ncells_all:
            with torch.cuda.stream(self.side):
                self.feat[slot].copy_(self.feat_all)
        else:
            A.call("pg_cell_select", self._ptr(self.feat_all), self.ncells_all, self.ncells, self._ptr(self.feat[slot]),
                   self.side_h)
        if predict:
            self.predict_log(slot, stream=self.side_h)
            with torch.cuda.stream(self.side):
                self.result_host.copy_(self.result, non_blocking=True)
        self.ev_pred.record(self.side)
        self._side_busy = True
        self._next = slot
        return self.ev_pred

    def open_cycle(self, step):
        """Start the new cycle with the sample taken at its build."""
        if self._next is not None:
            self.pending.append((self._next, step))
            self._next = None
        self._open_start = step
        self._open_pred = None

    def _calibrated(self, raw_log):
        self._open_pred = raw_log
        return math.exp(raw_log + self.bias)

    def predicted(self):
        """Predicted steps of the new cycle (after the rebuild's status read)."""
        self._side_done()
        return self._calibrated(float(self.result_host[0]))

    def raw_prediction(self):
        """The network's log prediction for the new cycle, as read with the rebuild's
        status, and the calibrated number of steps (the bias as of the last closed
        cycle).  note_prediction() later records it for the cycle's calibration."""
        self._side_done()
        raw = float(self.result_host[0])
        return raw, math.exp(raw + self.bias)

    def note_prediction(self, raw_log):
        self._open_pred = raw_log

    def _calibrate(self, trip_step, end_step):
        """Move the bias towards log(observed / predicted) of the cycle that closes: a
        trip gives the length, a cycle ended before any trip only a lower bound (which
        can raise the bias, never lower it)."""
        if self._open_pred is None or self._open_start is None:
            return
        if trip_step is not None:
            err = math.log(max(trip_step - self._open_start, 1)) - self._open_pred
            self.bias += self.calib_rate * (err - self.bias)
        else:
            err = math.log(max(end_step - self._open_start, 1)) - self._open_pred
            if err > self.bias:
                self.bias += self.calib_rate * (err - self.bias)

    def close_cycle(self, trip_step, end_step):
        """Label the open cycle: tripped at trip_step (exact), or censored at end_step."""
        self._calibrate(trip_step, end_step)
        for slot, step in self.pending:
            if trip_step is not None:
                r = max(trip_step - step, 1)
                self.labels.append((slot, math.log(r), 0))
            else:
                r = max(end_step - step, 1)
                self.labels.append((slot, math.log(r), 1))
        self.pending = []
        self.cycles += 1
        if self.trained and self.online_every and self.cycles % self.online_every == 0:
            self.train(self.online_steps, recent=self.online_recent, log=False)

    # ---------------------------------------------------------------- training
    def train(self, steps=None, recent=None, log=True):
        """Adam steps on the stored samples (the `recent` newest ones if given).  With
        log, the final loss is read back (a host sync) and returned."""
        e = self.e
        steps = self.train_steps if steps is None else steps
        if not self.labels:
            return None
        batch = self.labels if recent is None else self.labels[-recent:]
        ns = len(batch)
        # on the side stream, beside the steps; after the engine's stream has written the
        # samples (mid-cycle features are taken there)
        self.ev_feat.record(e.stream)
        self.side.wait_event(self.ev_feat)
        with torch.cuda.stream(self.side):
            for _ in range(steps):
                self.loss.zero_()
                for slot, target, cens in batch:
                    self.predict_log(slot, stream=self.side_h)
                    A.call("pg_mlp_backward", self._ptr(self.params), self._ptr(self.feat[slot]),
                           self._ptr(self.out), self.ncells, self._ptr(self.result), float(target), int(cens),
                           self.temperature, self._ptr(self.grads), self._ptr(self.loss), self.side_h)
                self.adam_t += 1
                A.call("pg_mlp_adam", self._ptr(self.params), self._ptr(self.grads), self._ptr(self.m1),
                       self._ptr(self.m2), self.lr, 0.9, 0.999, 1e-8, self.adam_t, 1.0 / ns, self.side_h)
        self.ev_pred.record(self.side)
        self._side_busy = True
        self.trained = True
        if not log:
            return None
        self.ev_pred.synchronize()
        final = float(self.loss.item()) / ns
        self.train_log.append(final)
        return final

    def predicted_steps(self):
        """Predict R for the current state (features at since_build) -> float steps."""
        slot = self._slot()
        self.features_into(slot)
        self.predict_log(slot)
        return self._calibrated(float(self.result[0].item())), slot


class EMASchedule:
    """Policy "ema": the trivial predictor the learned schedule is measured against.

    It predicts the next cycle's length (steps from a list build to the first guard
    trip) as an exponential moving average of the lengths seen so far, with no GPU
    work at all.  A cycle that ended at a proactive rebuild before any trip only
    bounds its length from below, so such a cycle can raise the average but never
    lower it.  Stepping, speculation, rewinds and the exact FP64 guard are the
    learned policy's; only the prediction differs.
    """

    samples_per_cycle = 0

    def __init__(self, engine, alpha=0.3, margin=1.2, warmup_cycles=3):
        self.e = engine
        self.alpha = alpha
        # a step past the trip costs only its skipped launches, a rebuild before the
        # trip a whole list build: the margin leans towards running past the trip
        self.margin = margin
        self.warmup_cycles = warmup_cycles
        self.ema = None
        self.cycles = 0
        self.trained = False
        self.pending = []
        self.history = []
        self._next = None
        self._start = None

    def sample_after_bin(self, predict):
        self._next = 0
        return None

    def open_cycle(self, step):
        self._start = step
        self._next = None

    def record(self, step):
        pass

    def close_cycle(self, trip_step, end_step):
        if self._start is None:
            return
        if trip_step is not None:
            length = max(trip_step - self._start, 1)
            self.ema = length if self.ema is None else (1 - self.alpha) * self.ema + self.alpha * length
        else:
            length = max(end_step - self._start, 1)
            blend = length if self.ema is None else (1 - self.alpha) * self.ema + self.alpha * length
            self.ema = blend if self.ema is None else max(self.ema, blend)
        self.cycles += 1

    def train(self, *args, **kw):
        self.trained = self.ema is not None
        return None

    def predicted(self):
        return self.ema

    def predicted_steps(self):
        return self.ema, None
