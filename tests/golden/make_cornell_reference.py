"""Makes tests/golden/cornell256_oracle_16k.npz: the CPU oracle's 16384-spp
render of the 256 x 256 Cornell room (depth 5, Russian roulette after bounce
3, box filter), the reference image of the GPU convergence test.

32 passes of 512 spp (stratified 32 x 16), each rendered into a float64 film
(the oracle's tile and film sums in double precision).  Seed 99: the GPU test
renders with other seeds, so the two share no random numbers.  The fixture
holds, per pixel, the mean of the 32 pass estimates (X, Y, Z) / weight and
the variance of that mean (from the spread of the passes), as float32.

    python tests/golden/make_cornell_reference.py [threads]

It takes about an hour on 8 cores.
"""
from __future__ import annotations

import sys
import time
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
ROOT = HERE.parents[1]
if str(ROOT) not in sys.path:
    sys.path.insert(0, str(ROOT))

from bling_gb300 import scene as S  # noqa: E402
from oracle.oracle import OracleScene  # noqa: E402

OUT = HERE / "cornell256_oracle_16k.npz"
SIZE, PASSES, STRATA, SEED = 256, 32, (32, 16), 99


def main(argv):
    nth = int(argv[1]) if len(argv) > 1 else 0
    sc = S.cornell_room(SIZE, SIZE)
    base = S.cornell_params(SIZE, SIZE)
    p = S.render_params(SIZE, SIZE, STRATA, max_depth=base.max_depth,
                        sample_depth=base.sample_depth, rr_depth=base.rr_depth,
                        filter_kind=base.filter_kind, seed=SEED)
    o = OracleScene(sc)
    est = []
    t0 = time.time()
    for k in range(PASSES):
        film, _ = o.render_pass_f64(p, k, nthreads=nth)
        est.append(film[..., 1:] / film[..., :1])
        print(f"pass {k + 1}/{PASSES}  {time.time() - t0:.0f} s", flush=True)
    e = np.stack(est)
    mean = e.mean(0)
    var_mean = e.var(0, ddof=1) / PASSES
    np.savez_compressed(OUT, mean=mean.astype(np.float32), var_mean=var_mean.astype(np.float32),
                        spp=np.int64(PASSES * STRATA[0] * STRATA[1]), passes=np.int64(PASSES),
                        seed=np.int64(SEED))
    print("wrote", OUT)


if __name__ == "__main__":
    main(sys.argv)
