"""Producer/consumer batch driver (emsim/simulator.py:21-91).

A producer thread iterates the molecules, a consumer thread runs the pipe on each and
the calling thread hands every result to ``result_handler`` as a numpy array (device
results are copied with ``.get()``).  A failing molecule is logged and skipped.
"""
from __future__ import annotations

import logging
import sys
import time
from queue import Queue
from threading import Event, Thread
from typing import Callable, Iterable

import numpy as np

from . import atoms as atm
from . import pipe

logger = logging.getLogger(__name__)


class ImagePipeRunFailed(Exception):
    pass


class EMSim:
    def __init__(self, image_pipe: pipe.Pipe, mols: Iterable[atm.AtomList], result_handler: Callable):
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
            for mol in self.mols_iter:
                if self.stop_event.is_set():
                    return
                self._task_q.put(mol)
        except Exception as e:  # a failing molecule source ends the run after reporting
            self._task_q.put(e)
        self._task_q.put(None)

    def consumer(self):
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
