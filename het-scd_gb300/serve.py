"""Served SCD: a continuous-batching request loop over the batched engine.

Requests (one edge list each) are admitted into batches while the device
works on earlier ones:

* admission control: a request is admitted only while the estimated device
  memory of all admitted, unfinished requests stays under the HBM budget
  (120 GB by default); the estimate is bytes_per_record x records, measured
  for this engine (the preprocessing keys and the resident graph dominate);
* continuous batching: `workers` engine contexts, each with its own CUDA
  stream, run on their own host threads (the C calls release the GIL).  A
  worker that becomes free takes every admitted request that is waiting (up to
  `max_batch`) as one block-diagonal batch, so requests that arrive while
  other batches are on the GPU start as soon as a slot and memory free up,
  and their work overlaps on the device with the batches still running;
* results: the best labels, WCC and iteration count of each request are
  exactly those of processing that request alone (the batched engine keeps
  all per-graph arithmetic per graph).

Latency of a request = time from submission to its labels being on the host.
"""
import collections
import threading
import time

import numpy as np

import scd_gb300 as S

BYTES_PER_RECORD = 96   # device bytes per input edge record at the preprocessing peak


class Request:
    __slots__ = ("pairs", "records", "submitted", "started", "finished", "result", "labels", "error",
                 "done", "id")

    def __init__(self, rid, pairs):
        self.id = rid
        self.pairs = np.ascontiguousarray(pairs, dtype=np.uint32).reshape(-1, 2)
        self.records = self.pairs.shape[0]
        self.submitted = time.perf_counter()
        self.started = self.finished = None
        self.result = self.labels = self.error = None
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
    def __init__(self, device=0, workers=4, budget_bytes=120e9, max_batch=64, threshold=0.01, max_iters=1000,
                 bytes_per_record=BYTES_PER_RECORD, engine_factory=None):
        self.budget = float(budget_bytes)
        self.max_batch = max_batch
        self.threshold = threshold
        self.max_iters = max_iters
        self.bytes_per_record = bytes_per_record
        self._lock = threading.Condition()
        self._waiting = collections.deque()
        self._in_use = 0.0
        self._closing = False
        self._next_id = 0
        self.batches = []          # (size, seconds) of every batch run
        self.peak_in_use = 0.0
        make = engine_factory or (lambda: S.Engine(device))
        self._engines = [make() for _ in range(workers)]
        self._threads = [threading.Thread(target=self._work, args=(e,), daemon=True) for e in self._engines]
        for t in self._threads:
            t.start()

    def cost(self, records):
        return max(records, 1) * self.bytes_per_record + 64e6

    def submit(self, pairs):
        with self._lock:
            req = Request(self._next_id, pairs)
            self._next_id += 1
            if self.cost(req.records) > self.budget:
                req.error = S.ScdError(-3, "request larger than the whole HBM budget")
                req.finished = time.perf_counter()
                req.done.set()
                return req
            self._waiting.append(req)
            self._lock.notify_all()
        return req

    def _take_batch(self):
        """Admitted waiting requests that fit the budget (FIFO, no overtaking)."""
        batch = []
        while self._waiting and len(batch) < self.max_batch:
            c = self.cost(self._waiting[0].records)
            if self._in_use + c > self.budget:
                break
            self._in_use += c
            batch.append(self._waiting.popleft())
        self.peak_in_use = max(self.peak_in_use, self._in_use)
        return batch

    def _work(self, eng):
        while True:
            with self._lock:
                while not self._closing and not self._waiting:
                    self._lock.wait()
                if self._closing and not self._waiting:
                    return
                batch = self._take_batch()
                if not batch:   # budget exhausted: wait for a finishing batch
                    self._lock.wait(0.01)
                    continue
            t0 = time.perf_counter()
            for r in batch:
                r.started = t0
            try:
                eng.batch_convert([r.pairs for r in batch])
                results, rc = eng.batch_run(self.threshold, self.max_iters)
                labels = eng.batch_labels_all()
                for g, r in enumerate(batch):
                    r.result = results[g]
                    r.labels = labels[g]
            except Exception as e:   # the batch fails as a whole; report it on every request
                for r in batch:
                    r.error = e
            t1 = time.perf_counter()
            with self._lock:
                self._in_use -= sum(self.cost(r.records) for r in batch)
                self.batches.append((len(batch), t1 - t0))
                self._lock.notify_all()
            for r in batch:
                r.finished = t1
                r.done.set()

    def close(self):
        with self._lock:
            self._closing = True
            self._lock.notify_all()
        for t in self._threads:
            t.join()
        for e in self._engines:
            e.close()

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
