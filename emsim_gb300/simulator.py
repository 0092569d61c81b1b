"""Producer/consumer batch driver (emsim/simulator.py:21-91).

A producer thread iterates the molecules, a consumer thread runs the pipe on each and
the calling thread hands every result to ``result_handler`` as a numpy array (device
results are copied with ``.get()``).  A failing molecule is logged and skipped.

``batch_size`` > 1 (an addition; the reference images one molecule at a time): the
consumer groups that many molecules and keeps two groups in flight through
``Pipe.submit_batch``, so the host stages one group while the GPU images the other.
Results still reach the handler in input order, one per molecule.  A group that fails
as a whole is run again molecule by molecule, so only the failing molecules are
reported, as with ``batch_size`` 1.

``shard=(rank, world)`` (an addition): one process per GPU, each running its own EMSim
over the same molecule source; rank r images the molecules i with i % world == r and
hands them to its own handler.  A stream of unknown length cannot be partitioned by
cost, so the split is round robin; ``Pipe.run_sharded`` balances a known list by cost.
"""
from __future__ import annotations

import logging
import sys
import time
from queue import Queue
from threading import Event, Thread
from typing import Callable, Iterable, List

import numpy as np

from . import atoms as atm
from . import pipe

logger = logging.getLogger(__name__)


class ImagePipeRunFailed(Exception):
    pass


class EMSim:
    def __init__(self, image_pipe: pipe.Pipe, mols: Iterable[atm.AtomList], result_handler: Callable,
                 batch_size: int = 1, shard=None):
        if batch_size < 1:
            raise ValueError("batch_size must be at least 1")
        if shard is not None:
            rank, world = (int(v) for v in shard)
            if world < 1 or not 0 <= rank < world:
                raise ValueError("shard must be (rank, world) with 0 <= rank < world")
            shard = (rank, world)
        self.shard = shard
        self.batch_size = int(batch_size)
        self.result_handler = result_handler
        self.image_pipe = image_pipe
        self.mols_iter = iter(mols)
        self.stop_event = Event()
        self._task_q: Queue = Queue()
        self._result_q: Queue = Queue()
        self._producer_thread = Thread(target=self.producer, daemon=True)
        self._consumer_thread = Thread(target=self.consumer, daemon=True)
        self.errors = []

    def run(self):
        self._producer_thread.start()
        self._consumer_thread.start()
        i = 0
        while True:
            try:
                i += 1
                result, label = self._result_q.get()
                if result is None and label == "done":
                    break
                if isinstance(result, Exception) and label == "error":
                    self.errors.append(result)
                    logger.warning(f"#{i} image run failed with {type(result)}: {str(result)}")
                elif isinstance(result, np.ndarray):
                    self.result_handler(result, label)
                else:
                    self.result_handler(result.get(), label)
            except (KeyboardInterrupt, SystemExit):
                print("exit signal received, waiting for threads to finish...")
                self.stop_event.set()
                self._producer_thread.join()
                self._consumer_thread.join()
                sys.exit("exit successfully.")
        logger.debug("all tasks done")

    def producer(self):
        try:
            for i, mol in enumerate(self.mols_iter):
                if self.stop_event.is_set():
                    return
                if self.shard is not None and i % self.shard[1] != self.shard[0]:
                    continue  # another rank's molecule
                self._task_q.put(mol)
        except Exception as e:  # a failing molecule source ends the run after reporting
            self._task_q.put(e)
        self._task_q.put(None)

    def consumer(self):
        if self.batch_size > 1 and hasattr(self.image_pipe, "submit_batch"):
            return self._consumer_batched()
        counter = 0
        while not self.stop_event.is_set():
            task = self._task_q.get()
            if task is None:
                self._result_q.put((None, "done"))
                return
            if isinstance(task, Exception):
                self._result_q.put((task, "error"))
                continue
            label = getattr(task, "label", None)
            start = time.perf_counter()
            try:
                result = self.image_pipe.run(task)
            except Exception as e:
                self._result_q.put((e, "error"))
            else:
                self._result_q.put((result, label))
            counter += 1
            logger.info(f"emsim: {counter} images processed, label = {label}, "
                        f"time elapsed = {time.perf_counter() - start:.3f}")

    def _run_one(self, mol):
        try:
            result = self.image_pipe.run(mol)
        except Exception as e:
            self._result_q.put((e, "error"))
        else:
            self._result_q.put((result, getattr(mol, "label", None)))

    def _consumer_batched(self):
        batch: List = []
        in_flight = None  # (pending images or None when the submission failed, molecules)
        counter = 0

        def collect(entry):
            nonlocal counter
            pending, mols = entry
            start = time.perf_counter()
            imgs = None
            if pending is not None:
                try:
                    imgs = pending.result()
                except Exception:
                    imgs = None
            if imgs is None:  # the group failed as a whole: find the failing molecules
                for mol in mols:
                    self._run_one(mol)
            else:
                for mol, img in zip(mols, imgs):
                    self._result_q.put((img, getattr(mol, "label", None)))
            counter += len(mols)
            logger.info(f"emsim: {counter} images processed, group of {len(mols)}, "
                        f"time waited = {time.perf_counter() - start:.3f}")

        def launch(mols):
            nonlocal in_flight
            try:
                entry = (self.image_pipe.submit_batch(mols), mols)
            except Exception:
                entry = (None, mols)
            if in_flight is not None:
                collect(in_flight)  # the earlier group first: results stay in input order
            in_flight = entry

        while not self.stop_event.is_set():
            task = self._task_q.get()
            if task is None or isinstance(task, Exception):
                if batch:
                    launch(batch)
                    batch = []
                if in_flight is not None:
                    collect(in_flight)
                    in_flight = None
                if task is None:
                    self._result_q.put((None, "done"))
                    return
                self._result_q.put((task, "error"))
                continue
            batch.append(task)
            if len(batch) == self.batch_size:
                launch(batch)
                batch = []
