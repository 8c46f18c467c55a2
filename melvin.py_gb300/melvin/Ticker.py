"""Cadence callbacks (melvin/Ticker.py): fire ``fn(ticker)`` once the loop
counter (or simulation time) passes the next multiple of ``cadence``."""


class Ticker:
    def __init__(self, cadence, fn, dump_name="", is_loop_counter=True):
        self._cadence = cadence
        self._fn = fn
        self._counter = 0
        self.times_fired = 0
        self._dump_name = dump_name
        self._by_counter = is_loop_counter

    def tick(self, t, loop_counter):
        now = loop_counter if self._by_counter else t
        if self._counter < now:
            self._fn(self)
            self._counter += self._cadence
            self.times_fired += 1

    def dump(self):
        return {"counter": self._counter, "times_fired": self.times_fired}

    def restore(self, data):
        self._counter = data["counter"]
        self.times_fired = data["times_fired"]

    def get_name(self):
        return self._dump_name
