"""Served SCD: continuous batching at the iteration level over a resident set.

Requests (one edge list each) join a set of graphs that stay resident on the
device and iterate together:

* admission control: a request is admitted only while the estimated device
  memory of all admitted, unfinished requests stays under the HBM budget
  (120 GB by default); the estimate is bytes_per_record x records, measured for
  this engine (the preprocessing keys and the resident graph dominate);
* conversion: `converters` staging engines, each on its own CUDA stream and
  host thread (the C calls release the GIL), take the admitted waiting requests
  (up to `max_batch`, FIFO) and preprocess them as one batch while the set
  iterates, then hand the graphs over (scd_resident_add);
* iteration: one host thread steps the resident set (scd_resident_step): every
  step is one refinement iteration of every running graph in the same launches
  (one CUDA-graph replay), so a request admitted while others are iterating
  joins their launches at the next step instead of waiting for a free worker;
  graphs that converge leave (scd_resident_take), which frees their share of
  the budget for the next admissions;
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


class Server:
    def __init__(self, device=0, converters=2, budget_bytes=120e9, max_batch=64, threshold=0.01, max_iters=1000,
                 bytes_per_record=BYTES_PER_RECORD, engine_factory=None, step_hook=None):
        """step_hook (optional): called with the number of steps made so far before
        every step of the resident set, on the iterating thread; it may block to
        hold the iterations (draining, or a test that lines up arrivals)."""
        self.budget = float(budget_bytes)
        self.max_batch = max_batch
        self.bytes_per_record = bytes_per_record
        self._lock = threading.Condition()
        self._waiting = collections.deque()
        self._in_set = {}           # resident-set id -> request (converted, not yet taken)
        self._in_use = 0.0
        self._closing = False
        self._failed = None
        self._next_id = 0
        self.batches = []           # (size, seconds) of every conversion batch
        self.step_running = []      # graphs that iterated in each step
        self.peak_in_use = 0.0
        self._step_hook = step_hook
        self._steps = 0
        make = engine_factory or (lambda: S.Engine(device))
        self.set = make()
        self.set.resident_init(threshold, max_iters)
        self._staging = [make() for _ in range(converters)]
        self._threads = [threading.Thread(target=self._convert, args=(e,), daemon=True) for e in self._staging]
        self._threads.append(threading.Thread(target=self._iterate, daemon=True))
        for t in self._threads:
            t.start()

    def cost(self, records):
        return max(records, 1) * self.bytes_per_record + 64e6

    def submit(self, pairs):
        with self._lock:
            req = Request(self._next_id, pairs)
            self._next_id += 1
            if self.cost(req.records) > self.budget:
                self._finish(req, S.ScdError(-3, "request larger than the whole HBM budget"))
                return req
            self._waiting.append(req)
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
            if req in self._waiting:
                self._waiting.remove(req)
                self._finish(req, Cancelled("request cancelled"))
            return True

    @staticmethod
    def _finish(req, error=None):
        req.error = error
        req.finished = time.perf_counter()
        req.done.set()

    def _take_batch(self):
        """Admitted waiting requests that fit the budget (FIFO, no overtaking)."""
        batch = []
        while self._waiting and len(batch) < self.max_batch:
            c = self.cost(self._waiting[0].records)
            if self._in_use + c > self.budget:
                break
            self._in_use += c
            r = self._waiting.popleft()
            r.admitted = True
            batch.append(r)
        self.peak_in_use = max(self.peak_in_use, self._in_use)
        return batch

    def _release(self, reqs):
        self._in_use -= sum(self.cost(r.records) for r in reqs)
        self._lock.notify_all()

    def _convert(self, eng):
        while True:
            with self._lock:
                while not self._closing and not self._waiting:
                    self._lock.wait()
                if self._closing and not self._waiting:
                    return
                batch = self._take_batch()
                if not batch:   # budget exhausted: wait for graphs to leave the set
                    self._lock.wait(0.01)
                    continue
            t0 = time.perf_counter()
            for r in batch:
                r.started = t0
            try:
                eng.batch_convert([r.pairs for r in batch])
                ids = self.set.resident_add(eng)
            except Exception as e:   # the batch fails as a whole; report it on every request
                with self._lock:
                    self._release(batch)
                for r in batch:
                    self._finish(r, e)
                continue
            with self._lock:
                for i, r in zip(ids, batch):
                    self._in_set[i] = r
                self.batches.append((len(batch), time.perf_counter() - t0))
                self._lock.notify_all()

    def _iterate(self):
        while True:
            with self._lock:
                while not self._in_set and not (self._closing and not self._waiting and self._converters_idle()):
                    self._lock.wait(0.05)
                if not self._in_set:
                    return
            if self._step_hook:
                self._step_hook(self._steps)
            self._steps += 1
            try:
                running, finished = self.set.resident_step()
                if running:
                    self.step_running.append(running)
                out = self.set.resident_take() if finished else []
            except Exception as e:   # the set is unusable: fail everything it holds
                with self._lock:
                    reqs = list(self._in_set.values())
                    self._in_set.clear()
                    self._release(reqs)
                for r in reqs:
                    self._finish(r, e)
                continue
            if not out:
                continue
            with self._lock:
                done = [(self._in_set.pop(i), res, st, lab) for i, res, st, lab in out]
                self._release([r for r, *_ in done])
            for r, res, st, lab in done:
                if r.cancelled:
                    self._finish(r, Cancelled("request cancelled"))
                    continue
                r.result = res
                r.labels = lab
                self._finish(r, S.ScdError(st, "max_iters reached before convergence") if st else None)

    def _converters_idle(self):
        return all(not t.is_alive() for t in self._threads[:-1])

    def close(self):
        with self._lock:
            self._closing = True
            self._lock.notify_all()
        for t in self._threads:
            t.join()
        for e in self._staging:
            e.close()
        self.set.close()

    def mean_coscheduled(self):
        return float(np.mean(self.step_running)) if self.step_running else 0.0

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
