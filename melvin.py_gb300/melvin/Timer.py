"""Wall-clock split timer (melvin/Timer.py)."""

import time


class Timer:
    def __init__(self):
        self._start_time = 0.0
        self.diff = 0.0

    def start(self):
        self._start_time = time.time()

    def split(self):
        now = time.time()
        self.diff = now - self._start_time
        self._start_time = now
