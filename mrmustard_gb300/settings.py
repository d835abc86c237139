"""Run-time flags of the GB300 Hermite path.

``STABLE_FOCK_CONVERSION`` mirrors the reference's flag of the same name
(mrmustard/utils/settings.py:101): when true, ``hermite_renormalized`` uses the stable
(all-pivot average) recurrence even if ``stable=False`` is passed
(mrmustard/math/backend_manager.py:682).

``AUTOSHAPE_PROBABILITY``, ``AUTOSHAPE_MAX``, ``AUTOSHAPE_MIN`` mirror the reference's autoshape
defaults (mrmustard/utils/settings.py:67-74): the probability mass to capture per mode and the
clip range of the cutoffs, used when ``autoshape_numba``'s arguments are None.

``CHECK_DEVICE_STATUS``: after each call, synchronise and read the workspace status word, so a
bounded inter-CTA wait that gave up raises at the call that caused it.  Benchmarks switch it
off inside timed loops and check once afterwards.
"""

from __future__ import annotations

from contextlib import contextmanager


class _Settings:
    def __init__(self):
        self.STABLE_FOCK_CONVERSION = False
        self.CHECK_DEVICE_STATUS = True
        self.AUTOSHAPE_PROBABILITY = 0.99999
        self.AUTOSHAPE_MAX = 50
        self.AUTOSHAPE_MIN = 1

    @contextmanager
    def __call__(self, **kwargs):
        old = {k: getattr(self, k) for k in kwargs}
        for k, v in kwargs.items():
            if not hasattr(self, k):
                raise AttributeError(f"unknown setting {k}")
            setattr(self, k, v)
        try:
            yield self
        finally:
            for k, v in old.items():
                setattr(self, k, v)


settings = _Settings()
