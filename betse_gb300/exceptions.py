"""Exception contract of the step.

BETSE raises ``betse.exceptions.BetseSimUnstableException``
(``betse/exceptions.py:625``) when Vmem or a concentration becomes NaN. When
BETSE is importable that very class is re-exported, so callers that catch it
keep working; otherwise a stand-in with the same name is defined.
"""
from __future__ import annotations

try:  # pragma: no cover - depends on whether BETSE is installed
    from betse.exceptions import BetseSimUnstableException  # type: ignore
except Exception:  # noqa: BLE001
    class BetseSimUnstableException(RuntimeError):
        """The simulation became numerically unstable (NaN state)."""
