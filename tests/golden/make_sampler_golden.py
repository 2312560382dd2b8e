"""Regenerates tests/golden/samplers.npz: the samples the reference's own
UniformImageSampler and ClassWeightedImageSampler return on the images of
tests/cases.py:sampler_images(), for each configuration of SAMPLER_CONFIGS.

    make -C oracle ref REF=<Padenti source tree> && python tests/golden/make_sampler_golden.py

The samplers come from the Padenti sources compiled in place
(oracle/ref_shim/ref_sampler.cpp, over libstdc++'s mt19937, zlib's CRC-32 and
the two Boost distributions restated); the fixture lets the GPU machine, which has
no Padenti sources, check the CUDA samplers against them.
"""
from __future__ import annotations

import hashlib
import pathlib
import sys

import numpy as np

HERE = pathlib.Path(__file__).resolve().parent
sys.path.insert(0, str(HERE.parent.parent))
sys.path.insert(0, str(HERE.parent))

import oracle_bind as ob  # noqa: E402
from cases import SAMPLER_CONFIGS, sampler_images, sampler_weights  # noqa: E402


def main() -> None:
    if ob.ref("sampler") is None:
        raise SystemExit("oracle/_ref/libref_sampler.so missing: make -C oracle ref REF=<Padenti sources>")
    out = {}
    h = hashlib.sha256()
    for name, img_type, data, labels, k in sampler_images():
        h.update(np.ascontiguousarray(data).tobytes())
        h.update(np.ascontiguousarray(labels).tobytes())
        for cname, kind, ns, seed, rule in SAMPLER_CONFIGS:
            if kind == 1:
                got = ob.ref_sample_uniform(img_type, data, labels, ns, seed)
                if not (labels != 0).any():
                    continue  # the reference draws from an empty buffer
            else:
                got = ob.ref_sample_class_weighted(img_type, data, labels, ns, k, sampler_weights(rule, k), seed)
            out[f"{cname}/{name}"] = np.asarray(got, np.uint32)
    out["inputs_sha256"] = np.array(h.hexdigest())
    np.savez_compressed(HERE / "samplers.npz", **out)
    print(f"wrote {len(out) - 1} sample lists")


if __name__ == "__main__":
    main()
