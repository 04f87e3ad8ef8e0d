"""Makes the example-scene fixtures under tests/golden/examples/.

Reads bling's example scene files (examples/*.bling of the reference
checkout), parses each with bling_gb300.blingfile and saves the parsed flat
scene with scene_fixture.save: the fixtures carry our own record of the
scene, not the file text.  The GPU tests render them, reduced in size, on the
GPU and on the CPU oracle.

Only `renderer { ... }` blocks are changed before parsing: every one is
dropped and a neutral sampler/path block appended.  Many of the examples
predate the reference's own renderer grammar (they write `stratified
xSamples 2 ySamples 2`, where RendererParser.hs:62-73 reads two bare
integers) and the tests choose their own sample counts and depths anyway.
The rest of each file is parsed as written.

    python tests/golden/make_example_scenes.py [<bling checkout>/examples]
"""
from __future__ import annotations

import re
import sys
from pathlib import Path

HERE = Path(__file__).resolve().parent
sys.path.insert(0, str(HERE))
import scene_fixture  # noqa: E402

from bling_gb300 import blingfile as B  # noqa: E402

DEFAULT_SOURCE = Path("/root/reference/examples")

# the examples whose scene content the GPU path renders
EXAMPLES = ["blackbody-emission", "bumpmap", "cellnoise", "cornell-box", "cornell-box-specular",
            "cornell-box-underwater", "ducky", "glass-torus", "heightmap", "matte-test",
            "plastic-test", "race", "substrate", "trans-matte"]

NEUTRAL_RENDERER = ("renderer { sampler sampled { sampler { stratified 1 1 } "
                    "integrator { path maxDepth 5 sampleDepth 3 } } }")


def neutral_renderer(text: str) -> str:
    """the file with its renderer blocks dropped and a neutral one appended
    (comments are dropped first so that braces in them do not count)"""
    text = "\n".join(line.split("#", 1)[0] for line in text.splitlines())
    out, i = [], 0
    while True:
        m = re.search(r"\brenderer\s*\{", text[i:])
        if not m:
            out.append(text[i:])
            break
        start, j, depth = i + m.start(), i + m.end(), 1
        while depth:
            depth += (text[j] == "{") - (text[j] == "}")
            j += 1
        out.append(text[i:start])
        i = j
    return "".join(out) + "\n" + NEUTRAL_RENDERER + "\n"


def parse_example(src: Path) -> B.Job:
    return B.parse(neutral_renderer(src.read_text()), src.parent)


def source_dir(argv=None) -> Path | None:
    d = Path(argv[1]) if argv and len(argv) > 1 else DEFAULT_SOURCE
    return d if d.is_dir() else None


def main(argv):
    src = source_dir(argv)
    if src is None:
        raise SystemExit("bling's examples directory not found; pass it as the first argument")
    out = HERE / "examples"
    out.mkdir(exist_ok=True)
    for name in EXAMPLES:
        job = parse_example(src / f"{name}.bling")
        # the fixture rebuilds the camera from its inputs: they must give the
        # camera the file made
        assert bytes(job.camera_for(job.width, job.height)) == bytes(job.scene.camera), name
        scene_fixture.save(job, out / f"{name}.npz", f"examples/{name}.bling")
        print(name, job.width, job.height, "triangles", job.scene.n_triangles, "shapes",
              len(job.scene.shapes), "lights", len(job.scene.lights))


if __name__ == "__main__":
    main(sys.argv)
