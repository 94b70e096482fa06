"""Text writers of the legacy jetshow drivers (``write_2dvector`` and
``write_vector``, src/utils.cpp:211-236): every value divided by ``scale``,
followed by a space, one image row per line (or one value per line), in the
C++ stream's default number formatting (six significant digits, ``%g``)."""
from __future__ import annotations

from typing import IO, Iterable, Sequence


def _fmt(x: float) -> str:
    return "%g" % x


def write_2dvector(f: IO[str], image: Sequence[Sequence[float]], scale: float = 1.0) -> None:
    """image[i][j] / scale, row i on line i (``map_*.txt`` of the drivers)."""
    for row in image:
        f.write("".join(_fmt(x / scale) + " " for x in row) + "\n")


def write_vector(f: IO[str], values: Iterable[float], scale: float = 1.0) -> None:
    """values[i] / scale, one per line (the stripe files of the drivers)."""
    for x in values:
        f.write(_fmt(x / scale) + " \n")
