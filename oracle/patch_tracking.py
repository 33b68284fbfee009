"""Build step of the reference harness (oracle/Makefile, target ref): writes
build-time copies of two reference headers into oracle/_ref/patched/.  The
copies never enter the repository.

src/tracking/tracking_parameters.hpp, with exactly one fix so that the header
parses without Intel IPP: its non-IPP DefaultTrackingParametersConfig alias
(tracking_parameters.hpp:47-56) lists the policies out of order
(ReshapeAndSum before Mixer) with a trailing comma; the copy lists them in the
order TrackingParametersConfig declares (Abs, Correlator, MatchedFilter,
Mixer, ReshapeAndSum, Upsampler).

src/measurements/observable.hpp, unchanged but for access: its constructor
from a TrackingParameters history (observable.hpp:75-88) is private (only
FindPreambleGps / FindPreambleGlonass reach it, after decoding a whole
navigation message), so the copy opens the class with `public:`; its include
of tracking_parameters.hpp resolves to the fixed copy above.

Every other relative include is pointed back at the reference tree.

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

    obs = (ref / "src" / "measurements" / "observable.hpp").read_text()
    head = "\tclass Observable final {\n"
    if obs.count(head) != 1:
        raise SystemExit("observable.hpp: the class head is not the expected text")
    obs = obs.replace(head, head + "\tpublic:  // build-time copy: the constructor is reachable from the harness\n")
    obs = obs.replace('#include "../tracking/tracking_parameters.hpp"', f'#include "{dst.resolve()}/tracking_parameters.hpp"')
    obs = re.sub(r'#include "\.\./', f'#include "{ref / "src"}/', obs)
    obs = re.sub(r'#include "(timescale\.hpp)"', f'#include "{ref / "src" / "measurements"}/\\1"', obs)
    mdst = out / "patched" / "measurements"
    mdst.mkdir(parents=True, exist_ok=True)
    (mdst / "observable.hpp").write_text(obs)


if __name__ == "__main__":
    main()
