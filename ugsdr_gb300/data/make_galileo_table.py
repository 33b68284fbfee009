"""Writes galileo_e1_memory_codes.bin: the Galileo E1B and E1C primary codes
(Galileo OS SIS ICD memory codes, 50 codes of 4,092 chips per signal) as
packed bits, from tests/golden/codes.npz (which the reference's own
PrnGenerator<Galileo_E1b / Galileo_E1c>::Get produced as BOC(1,1) half-chips
[c, -c]).  Layout: E1B codes 0..49 then E1C codes 0..49, each 512 bytes,
chip i in byte i // 8 at bit 7 - i % 8, bit 1 = chip value -1.  The library
embeds the file at build time (ugsdr_gb300/build.py) and serves the codes
through ugsdr_prn_code."""
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent


def main() -> None:
    z = np.load(HERE.parents[1] / "tests" / "golden" / "codes.npz")
    blobs = []
    for name in ("galileo_e1b", "galileo_e1c"):
        n = int(z[name + "_len"])
        half = np.unpackbits(z[name], axis=1)[:, :n]
        chips = half[:, 0::2]                       # bit of c in each [c, -c] pair
        assert np.array_equal(half[:, 1::2], 1 - chips) and chips.shape == (50, 4092)
        padded = np.zeros((50, 4096), np.uint8)
        padded[:, :4092] = chips
        blobs.append(np.packbits(padded, axis=1))
    data = np.concatenate(blobs).tobytes()
    assert len(data) == 2 * 50 * 512
    (HERE / "galileo_e1_memory_codes.bin").write_bytes(data)


if __name__ == "__main__":
    main()
