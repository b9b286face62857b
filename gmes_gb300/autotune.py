"""Launch-shape autotuner for the multi-grid (batch) kernels.

The batch update kernel has two shape knobs: the block's extent along k
(``bx_cap``: 2**bx_cap threads along k, the rest along j) and the grid size
of the persistent kernel (``blocks``; 0 = one block per tile).  Which is
best depends on the mix of grid shapes (thin 2-D grids want short k extents,
large 3-D grids want full warps along k and enough blocks to hide memory
latency).  The tuner measures candidates on live chunks -- every candidate
computes exactly the same values, so tuning costs no extra work -- timing
each chunk on the device (CUDA events around its launches on the batch's
stream), and keeps the fastest per mix bucket.
"""


def _sms():
    from .engine import _torch
    torch = _torch()
    return torch.cuda.get_device_properties(torch.cuda.current_device()).multi_processor_count


class Tuner:
    """Per-bucket choice of (bx_cap, blocks) from measured chunk throughput."""

    def __init__(self, candidates=None, trials_per_candidate=1):
        sms = _sms()
        # block extent along k (2^bx_cap cells) x persistent grid size
        # (0: one block per tile; else a multiple of the SM count)
        self.candidates = candidates or [
            (bx, blocks) for bx in (4, 5, 3) for blocks in (0, 12 * sms, 24 * sms, 48 * sms)]
        self.trials_per_candidate = int(trials_per_candidate)
        self.best = {}
        self.results = {}
        self._key = None
        self._cand = None
        self._ev = None

    @staticmethod
    def bucket(jobs):
        """Mix bucket: number of grids (power of 2), dimensionality, size scale."""
        n = len(jobs)
        nb = 1
        while nb < n:
            nb *= 2
        thin = sum(1 for j in jobs if j.scene.n[2] < 32)
        cells = sorted(j.scene.cells for j in jobs)
        med = cells[len(cells) // 2]
        scale = 0
        while (1 << (2 * scale + 10)) < med:
            scale += 1
        return (nb, "2d" if thin * 2 > n else "3d", scale)

    def choice(self, jobs):
        key = self.bucket(jobs)
        self._key = key
        if key in self.best:
            self._cand = self.best[key]
            return self._cand
        tried = self.results.setdefault(key, {})
        for cand in self.candidates:
            if len(tried.get(cand, [])) < self.trials_per_candidate:
                self._cand = cand
                return cand
        self.best[key] = max(tried, key=lambda c: max(tried[c]))
        self._cand = self.best[key]
        return self._cand

    def observe_start(self, batch):
        """Before a chunk's launches: a start event on the batch's stream
        (only while the bucket is still being explored)."""
        self._ev = None
        if self._key is None or self._key in self.best:
            return
        from .engine import _torch
        torch = _torch()
        self._ev = (torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True))
        self._ev[0].record(batch.stream)

    def observe_stop(self, batch):
        """After the chunk's launches: the end event."""
        if self._ev is not None:
            self._ev[1].record(batch.stream)

    def observe_end(self, batch, cell_updates):
        """After the chunk has completed: record its device-timed throughput."""
        if self._ev is None:
            return
        ms = self._ev[0].elapsed_time(self._ev[1])
        self._ev = None
        cand = (batch.bx_cap, batch.blocks)
        if ms > 0:
            self.results.setdefault(self._key, {}).setdefault(cand, []).append(
                cell_updates / (ms / 1e3))

    def summary(self):
        return {str(k): {"best": v, "measured": {str(c): max(r) for c, r in
                                                  self.results.get(k, {}).items()}}
                for k, v in self.best.items()}
