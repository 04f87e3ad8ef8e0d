"""Save and load parsed scenes as test fixtures (an .npz of our own flat
scene record; no scene file text).

A fixture holds what bling_gb300.blingfile.parse makes of a .bling file: the
materials (bling_material records as bytes), meshes (vertices, indices,
normals, uvs, material), shapes (kind, parameters, object-to-world transform
and its inverse, material, emission), lights (kind, spectrum, vector,
environment map, world-to-light transform, sun/sky east and turbidity), the
texture nodes (kind, children, mapping, numbers, spectrum, gradient steps,
image pixels), the primitive order, the camera inputs (camera-to-world, lens radius, focal
distance, field of view) and the
job's image size, filter, sampler and depths.
"""
from __future__ import annotations

import json
import sys
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parents[2]
if str(ROOT) not in sys.path:
    sys.path.insert(0, str(ROOT))

from bling_gb300 import abi  # noqa: E402
from bling_gb300 import blingfile as B  # noqa: E402
from bling_gb300 import scene as S  # noqa: E402
from bling_gb300 import transform as xf  # noqa: E402

FORMAT = 1


def save(job: B.Job, path: Path, source: str) -> None:
    sc = job.scene
    arrays = {}
    meta = {"format": FORMAT, "source": source, "width": job.width, "height": job.height,
            "filter_kind": job.filter_kind, "filter_params": [float(x) for x in job.filter_params],
            "renderer": job.renderer, "sampler_kind": job.sampler_kind,
            "strata": list(job.strata), "max_depth": job.max_depth,
            "sample_depth": job.sample_depth, "prim_order": list(map(int, sc.prim_order or [])),
            "meshes": [], "shapes": [], "lights": []}
    arrays["materials"] = np.frombuffer(b"".join(bytes(m) for m in sc.materials), np.uint8)
    meta["n_materials"] = len(sc.materials)
    for k, m in enumerate(sc.meshes):
        arrays[f"mesh{k}_v"] = m.vertices
        arrays[f"mesh{k}_i"] = m.indices
        if m.normals is not None:
            arrays[f"mesh{k}_n"] = m.normals
        if m.uvs is not None:
            arrays[f"mesh{k}_uv"] = m.uvs
        meta["meshes"].append({"material": m.material, "normals": m.normals is not None,
                               "uvs": m.uvs is not None})
    for k, s in enumerate(sc.shapes):
        arrays[f"shape{k}_xf"] = np.stack([s.o2w.m, s.o2w.inv])
        if s.emission is not None:
            arrays[f"shape{k}_e"] = s.emission
        meta["shapes"].append({"kind": s.kind, "params": [float(np.float32(p)) for p in s.params],
                               "material": s.material, "emission": s.emission is not None})
    for k, l in enumerate(sc.lights):
        arrays[f"light{k}_s"] = np.asarray(l.spectrum, np.float32)
        if l.env is not None:
            arrays[f"light{k}_env"] = np.asarray(l.env, np.float32)
        if l.w2l is not None:
            arrays[f"light{k}_xf"] = np.stack([l.w2l.m, l.w2l.inv])
        meta["lights"].append({"kind": l.kind, "vec": [float(np.float32(v)) for v in l.vec],
                               "env": l.env is not None, "w2l": l.w2l is not None,
                               "east": [float(np.float32(v)) for v in l.east],
                               "turbidity": float(np.float32(l.turbidity))})
    meta["textures"] = []
    for k, t in enumerate(sc.textures):
        if t.spectrum is not None:
            arrays[f"tex{k}_s"] = np.asarray(t.spectrum, np.float32)
        if t.steps is not None:
            arrays[f"tex{k}_steps"] = np.asarray(t.steps, np.float32)
        if t.pixels is not None:
            arrays[f"tex{k}_px"] = np.asarray(t.pixels, np.uint8)
        meta["textures"].append({"kind": t.kind, "children": list(map(int, t.children)),
                                 "ivalue": int(t.ivalue), "map_kind": int(t.mapping[0]),
                                 "map": [float(np.float32(x)) for x in t.mapping[1]],
                                 "p": [float(np.float32(x)) for x in t.p]})
    c2w, lr, fd, fov = job.camera_view
    arrays["camera_c2w"] = np.stack([c2w.m, c2w.inv])
    meta["camera"] = {"lens_radius": float(lr), "focal_distance": float(fd), "fov": float(fov)}
    arrays["meta"] = np.frombuffer(json.dumps(meta, sort_keys=True).encode(), np.uint8)
    np.savez_compressed(path, **arrays)


def load(path: Path) -> B.Job:
    z = np.load(path)
    meta = json.loads(bytes(z["meta"]).decode())
    assert meta["format"] == FORMAT
    sc = S.Scene()
    raw = z["materials"].tobytes()
    size = len(raw) // max(1, meta["n_materials"])
    sc.materials = [abi.Material.from_buffer_copy(raw[k * size:(k + 1) * size])
                    for k in range(meta["n_materials"])]
    for k, m in enumerate(meta["meshes"]):
        sc.add_mesh(z[f"mesh{k}_v"], z[f"mesh{k}_i"], m["material"],
                    normals=z[f"mesh{k}_n"] if m["normals"] else None,
                    uvs=z[f"mesh{k}_uv"] if m["uvs"] else None)
    for k, s in enumerate(meta["shapes"]):
        x = z[f"shape{k}_xf"]
        sc.add_shape(s["kind"], tuple(np.float32(p) for p in s["params"]),
                     xf.Transform(x[0], x[1]), s["material"],
                     emission=z[f"shape{k}_e"] if s["emission"] else None)
    for k, l in enumerate(meta["lights"]):
        x = z[f"light{k}_xf"] if l["w2l"] else None
        sc.lights.append(S.Light(l["kind"], z[f"light{k}_s"], tuple(l["vec"]),
                                 z[f"light{k}_env"] if l["env"] else None,
                                 xf.Transform(x[0], x[1]) if x is not None else None,
                                 east=tuple(l.get("east", (0.0, 0.0, 0.0))),
                                 turbidity=l.get("turbidity", 0.0)))
    for k, t in enumerate(meta.get("textures", [])):
        sc.textures.append(S.Texture(
            t["kind"], tuple(t["children"]), t["ivalue"],
            (t["map_kind"], tuple(np.float32(x) for x in t["map"])),
            tuple(np.float32(x) for x in t["p"]),
            z[f"tex{k}_s"] if f"tex{k}_s" in z else None,
            z[f"tex{k}_steps"] if f"tex{k}_steps" in z else None,
            z[f"tex{k}_px"] if f"tex{k}_px" in z else None))
    sc.prim_order = meta["prim_order"]
    c = z["camera_c2w"]
    cam = meta["camera"]
    view = (xf.Transform(c[0], c[1]), np.float32(cam["lens_radius"]),
            np.float32(cam["focal_distance"]), np.float32(cam["fov"]))
    job = B.Job(sc, meta["width"], meta["height"], meta["filter_kind"],
                tuple(meta["filter_params"]), meta["renderer"], meta["sampler_kind"],
                tuple(meta["strata"]), meta["max_depth"], meta["sample_depth"],
                camera_view=view)
    sc.camera = job.camera_for(job.width, job.height)
    return job


def fixtures() -> list[Path]:
    return sorted((Path(__file__).resolve().parent / "examples").glob("*.npz"))
