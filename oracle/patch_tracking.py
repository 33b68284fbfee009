"""Build step of the reference harness (oracle/Makefile, target ref): writes a
build-time copy of the reference's src/tracking/tracking_parameters.hpp into
oracle/_ref/patched/tracking/ with exactly one fix, so that the header parses
without Intel IPP.  Its non-IPP DefaultTrackingParametersConfig alias
(tracking_parameters.hpp:47-56) lists the policies out of order (ReshapeAndSum
before Mixer) with a trailing comma; the copy lists them in the order
TrackingParametersConfig declares (Abs, Correlator, MatchedFilter, Mixer,
ReshapeAndSum, Upsampler).  Relative includes are pointed back at the
reference tree.  Nothing else changes; the copy never enters the repository.

usage: python3 patch_tracking.py REF_DIR OUT_DIR"""
import re
import sys
from pathlib import Path

BROKEN = """		SequentialAbs,
		SequentialCorrelator,
		SequentialMatchedFilter,
		SequentialReshapeAndSum,
		TableMixer,
		
		SequentialUpsampler,
#endif"""
FIXED = """		SequentialAbs,
		SequentialCorrelator,
		SequentialMatchedFilter,
		TableMixer,
		SequentialReshapeAndSum,
		SequentialUpsampler
#endif"""


def main() -> None:
    ref, out = Path(sys.argv[1]).resolve(), Path(sys.argv[2])
    src = (ref / "src" / "tracking" / "tracking_parameters.hpp").read_text()
    if src.count(BROKEN) != 1:
        raise SystemExit("tracking_parameters.hpp: the non-IPP configuration alias is not the expected text")
    text = src.replace(BROKEN, FIXED)
    text = re.sub(r'#include "\.\./', f'#include "{ref / "src"}/', text)
    dst = out / "patched" / "tracking"
    dst.mkdir(parents=True, exist_ok=True)
    (dst / "tracking_parameters.hpp").write_text(text)


if __name__ == "__main__":
    main()
