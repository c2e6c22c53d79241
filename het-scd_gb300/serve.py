"""Served SCD: continuous batching at the iteration level over a resident set.

Requests (one edge list each) join a set of graphs that stay resident on the
device and iterate together:

* admission control: a request is admitted only while the estimated device
  memory of all admitted, unfinished requests stays under the HBM budget
  (120 GB by default); the estimate is bytes_per_record x records, measured for
  this engine (the preprocessing keys and the resident graph dominate);
* conversion: each lane has its own queue and `converters` staging engines,
  each on its own CUDA stream and host thread (the C calls release the GIL),
  which take the lane's admitted waiting requests (up to `max_batch`, FIFO) and
  preprocess them as one batch while the set iterates, then hand the graphs
  over (scd_resident_add); the first lane's engines (set and staging) run on
  high-priority streams, so small requests are not queued behind the thread
  blocks of large ones;
* iteration: each size lane (requests up to `lanes[0]` records, up to
  `lanes[1]`, ..., the rest) is one resident set stepped by its own host thread
  (scd_resident_step): every step is one refinement iteration of every running
  graph of the lane in the same launches (one CUDA-graph replay), so a request
  admitted while others are iterating joins their launches at the next step
  instead of waiting for a free worker; graphs that converge leave
  (scd_resident_take), which frees their share of the budget for the next
  admissions.  Lanes keep small requests from waiting on the iterations of
  large ones (and on the re-forming of a large union when graphs join); the
  lanes' launches overlap on the device;
* results: the best labels, WCC and iteration count of each request are those
  of processing that request alone (the resident set keeps every per-graph
  quantity per graph).

Latency of a request = time from submission to its labels being on the host.
A request can be cancelled: before its conversion it leaves the queue; after
it, its result is dropped when its graph leaves the set.
"""
import collections
import threading
import time

import numpy as np

import scd_gb300 as S

BYTES_PER_RECORD = 96   # device bytes per input edge record at the preprocessing peak


class Cancelled(RuntimeError):
    pass


class Request:
    __slots__ = ("pairs", "records", "submitted", "started", "finished", "result", "labels", "error",
                 "done", "id", "cancelled", "admitted")

    def __init__(self, rid, pairs):
        self.id = rid
        self.pairs = np.ascontiguousarray(pairs, dtype=np.uint32).reshape(-1, 2)
        self.records = self.pairs.shape[0]
        self.submitted = time.perf_counter()
        self.started = self.finished = None
        self.result = self.labels = self.error = None
        self.cancelled = False
        self.admitted = False
        self.done = threading.Event()

    @property
    def latency(self):
        return None if self.finished is None else self.finished - self.submitted

    def wait(self, timeout=None):
        if not self.done.wait(timeout):
            raise TimeoutError("request not finished")
        if self.error:
            raise self.error
        return self.result, self.labels


class Lane:
    """One resident set, its queue and staging engines, and the requests it holds
    (resident-set id -> request)."""

    def __init__(self, index, engine, staging, threshold, max_iters):
        self.index = index
        self.set = engine
        self.set.resident_init(threshold, max_iters)
        self.staging = staging
        self.waiting = collections.deque()
        self.in_set = {}
        self.step_running = []   # graphs that iterated in each step
        self.steps = 0
        self.converters = []


class Server:
    def __init__(self, device=0, converters=2, budget_bytes=120e9, max_batch=64, threshold=0.01, max_iters=1000,
                 bytes_per_record=BYTES_PER_RECORD, engine_factory=None, step_hook=None, lanes=(1 << 21,)):
        """lanes: ascending record-count bounds of the size lanes (one more lane
        takes the rest).  step_hook (optional): called with (lane index, steps the
        lane made so far) before every step, on the lane's thread; it may block to
        hold the iterations (draining, or a test that lines up arrivals)."""
        self.budget = float(budget_bytes)
        self.max_batch = max_batch
        self.bytes_per_record = bytes_per_record
        self._lock = threading.Condition()
        self._in_use = 0.0
        self._closing = False
        self._failed = None
        self._next_id = 0
        self.batches = []           # (size, seconds) of every conversion batch
        self.peak_in_use = 0.0
        self._step_hook = step_hook
        self.bounds = list(lanes)
        def make(high):
            if engine_factory:
                return engine_factory()
            return S.Engine(device, flags=S.FLAG_PRIORITY if high else 0)

        self.lanes = []
        for k in range(len(self.bounds) + 1):
            self.lanes.append(Lane(k, make(k == 0), [make(k == 0) for _ in range(converters)], threshold, max_iters))
        self._threads = []
        for ln in self.lanes:
            ln.converters = [threading.Thread(target=self._convert, args=(ln, e), daemon=True) for e in ln.staging]
            self._threads += ln.converters + [threading.Thread(target=self._iterate, args=(ln,), daemon=True)]
        for t in self._threads:
            t.start()

    @property
    def set(self):
        """The resident set of the first (smallest) lane."""
        return self.lanes[0].set

    @property
    def step_running(self):
        """Graphs that iterated in each step of the first lane."""
        return self.lanes[0].step_running

    def lane_of(self, records):
        return sum(records > b for b in self.bounds)

    def cost(self, records):
        return max(records, 1) * self.bytes_per_record + 64e6

    def submit(self, pairs):
        with self._lock:
            req = Request(self._next_id, pairs)
            self._next_id += 1
            if self.cost(req.records) > self.budget:
                self._finish(req, S.ScdError(-3, "request larger than the whole HBM budget"))
                return req
            self.lanes[self.lane_of(req.records)].waiting.append(req)
            self._lock.notify_all()
        return req

    def cancel(self, req):
        """Cancels a request: it leaves the queue if it was not converted yet; a
        converted one finishes its iterations on the device, but its result is
        dropped.  Either way it ends with a Cancelled error."""
        with self._lock:
            if req.done.is_set():
                return False
            req.cancelled = True
            waiting = self.lanes[self.lane_of(req.records)].waiting
            if req in waiting:
                waiting.remove(req)
                self._finish(req, Cancelled("request cancelled"))
            return True

    @staticmethod
    def _finish(req, error=None):
        req.error = error
        req.finished = time.perf_counter()
        req.done.set()

    def _take_batch(self, lane):
        """The lane's admitted waiting requests that fit the budget (FIFO, no overtaking)."""
        batch = []
        while lane.waiting and len(batch) < self.max_batch:
            c = self.cost(lane.waiting[0].records)
            if self._in_use + c > self.budget:
                break
            self._in_use += c
            r = lane.waiting.popleft()
            r.admitted = True
            r.started = time.perf_counter()   # under the lock: admission order
            batch.append(r)
        self.peak_in_use = max(self.peak_in_use, self._in_use)
        return batch

    def _release(self, reqs):
        self._in_use -= sum(self.cost(r.records) for r in reqs)
        self._lock.notify_all()

    def _convert(self, lane, eng):
        while True:
            with self._lock:
                while not self._closing and not lane.waiting:
                    self._lock.wait()
                if self._closing and not lane.waiting:
                    return
                batch = self._take_batch(lane)
                if not batch:   # budget exhausted: wait for graphs to leave the set
                    self._lock.wait(0.01)
                    continue
            t0 = time.perf_counter()
            try:
                eng.batch_convert([r.pairs for r in batch])
                ids = lane.set.resident_add(eng)
            except Exception as e:   # the batch fails as a whole; report it on every request
                with self._lock:
                    self._release(batch)
                for r in batch:
                    self._finish(r, e)
                continue
            with self._lock:
                for i, r in zip(ids, batch):
                    lane.in_set[i] = r
                self.batches.append((len(batch), time.perf_counter() - t0))
                self._lock.notify_all()

    def _iterate(self, lane):
        while True:
            with self._lock:
                while not lane.in_set and not (self._closing and not lane.waiting and self._converters_idle(lane)):
                    self._lock.wait(0.05)
                if not lane.in_set:
                    return
            if self._step_hook:
                self._step_hook(lane.index, lane.steps)
            lane.steps += 1
            try:
                running, finished = lane.set.resident_step()
                if running:
                    lane.step_running.append(running)
                out = lane.set.resident_take() if finished else []
            except Exception as e:   # the set is unusable: fail everything it holds
                with self._lock:
                    reqs = list(lane.in_set.values())
                    lane.in_set.clear()
                    self._release(reqs)
                for r in reqs:
                    self._finish(r, e)
                continue
            if not out:
                continue
            with self._lock:
                done = [(lane.in_set.pop(i), res, st, lab) for i, res, st, lab in out]
                self._release([r for r, *_ in done])
            for r, res, st, lab in done:
                if r.cancelled:
                    self._finish(r, Cancelled("request cancelled"))
                    continue
                r.result = res
                r.labels = lab
                self._finish(r, S.ScdError(st, "max_iters reached before convergence") if st else None)

    @staticmethod
    def _converters_idle(lane):
        return all(not t.is_alive() for t in lane.converters)

    def close(self):
        with self._lock:
            self._closing = True
            self._lock.notify_all()
        for t in self._threads:
            t.join()
        for ln in self.lanes:
            for e in ln.staging:
                e.close()
            ln.set.close()

    def mean_coscheduled(self):
        """Graphs per iteration step, over the steps of every lane."""
        steps = [x for ln in self.lanes for x in ln.step_running]
        return float(np.mean(steps)) if steps else 0.0

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()


def percentile(values, q):
    v = sorted(values)
    if not v:
        return None
    k = min(len(v) - 1, max(0, int(round(q / 100.0 * (len(v) - 1)))))
    return v[k]
