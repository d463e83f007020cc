"""Host-side data layouts shared with the C ABI (include/gbpt.h).

The scene records keep CudaPT's byte layouts so that a caller holding
reference data can pass it through unchanged:

* ``VERTEX``   -- ``RTVertex`` (include/raytracer.h:58-64): pos, norm, tan, tex; 44 bytes.
* ``TRIANGLE`` -- ``RTTriangle`` (include/raytracer.h:66-72): three vertex ids and a material id.
* ``MATERIAL`` -- ``RTMaterial`` (include/raytracer.h:82-101) without FULLSPECTRAL; 80 bytes.
* ``PARAMS``   -- ``gbpt_params``: the renderer knobs the reference kept as
  compile-time defines and GUI attributes.
"""
import numpy as np

VERTEX = np.dtype(
    [("pos", "<f4", 3), ("norm", "<f4", 3), ("tan", "<f4", 3), ("tex", "<f4", 2)], align=False
)
TRIANGLE = np.dtype([("v0", "<u4"), ("v1", "<u4"), ("v2", "<u4"), ("mat", "<u4")])
MATERIAL = np.dtype(
    [
        ("diffuse", "<f4", 3),
        ("emissive", "<f4", 3),
        ("diffuseTexId", "<i4"),
        ("normalTexId", "<i4"),
        ("emissiveTexId", "<i4"),
        ("matType", "<i4"),
        ("transparency", "<f4"),
        ("subsurface", "<f4"),
        ("specular", "<f4"),
        ("metallic", "<f4"),
        ("roughness", "<f4"),
        ("anisotropic", "<f4"),
        ("sheen", "<f4"),
        ("sheenTint", "<f4"),
        ("clearcoat", "<f4"),
        ("clearcoatGloss", "<f4"),
    ]
)
assert VERTEX.itemsize == 44 and TRIANGLE.itemsize == 16 and MATERIAL.itemsize == 80

PARAMS = np.dtype(
    [
        ("seed", "<u4"),
        ("eye_depth_max", "<u4"),
        ("light_depth_max", "<u4"),
        ("light_paths", "<u4"),
        ("light_every", "<u4"),
        ("env", "<f4", 3),
        ("warmup_frames", "<u4"),
        ("desired_n", "<u4"),
        ("filter_color_eud", "<f4"),
        ("filter_pos_eud", "<f4"),
        ("filter_norm_eud", "<f4"),
        ("filter_diff_eud", "<f4"),
        ("filter_radius", "<u4"),
        ("filter_diffuse", "<u4"),
        ("filter_sigma_spatial", "<f4"),
        ("request_id", "<u4"),
        ("min_trace_prob", "<f4"),
        ("bilat_color_eud", "<f4"),
        ("bilat_pos_eud", "<f4"),
        ("bilat_norm_eud", "<f4"),
        ("bilat_emit_eud", "<f4"),
        ("bilat_diff_eud", "<f4"),
        ("bilat_radius", "<u4"),
        ("filter_iterations", "<u4"),
        ("render_iterations", "<u4"),
        ("pt_depth_max", "<u4"),
        ("walk_refill", "<u4"),
        ("tail_from", "<i4"),
        ("bands", "<u4"),
        ("walk_ctas", "<u4"),
        ("carry_steps", "<u4"),
        ("tail_below", "<f4"),
    ]
)

# Renderer modes (the BDPT entries of the reference's X-macro list,
# include/raytracer.h:13-23).
MODE_BDPT_SC = 0              # "BDPTSC"                     cudaRTBDPTStream
MODE_BDPT_SC_ADAP_BILAT = 1   # "BDPTSC Adap Bilat PLL"      cudaRTBDPTStreamAdapBilatAtomic
MODE_BDPT_SC_ADAP_BILAT_BINARY = 2  # "BDPTSC Adap Bilat Binary"  cudaRTBDPTStreamAdapBilatBinary
MODE_BDPT_SC_BILAT = 3        # "BDPTSC Bilaterial"          cudaRTBDPTStreamBilat
MODE_PT_SC = 4                # "PTSC" (unidirectional)      cudaRTPTStream

# gbpt_read_buffer ids
BUF_RESULT, BUF_POS, BUF_NORM, BUF_DIFF, BUF_FILTERED, BUF_ERR, BUF_SAMPLE_N, BUF_LIGHT_CACHE = range(8)
BUF_DIRECT, BUF_EMIS, BUF_POTENTIAL = 8, 9, 10


def default_params(**over):
    """Reference defaults: depth caps 5/5 (src/cudaRTBDPTStream.cu:7,10),
    128 light paths every 3rd frame (:875-877), adaptive knobs of
    src/cudaRTBDPTStreamAdapBilatAtomic.cu:26-37, warm-up 5 frames (:1372),
    filter-only knobs of src/cudaRTBDPTStreamBilat.cu:29-37, PTSC depth cap 10
    (src/cudaRTPTStream.cu:6)."""
    p = np.zeros((), PARAMS)
    p["seed"] = 1234
    p["eye_depth_max"] = 5
    p["light_depth_max"] = 5
    p["light_paths"] = 128
    p["light_every"] = 3
    p["env"] = (0.0, 0.0, 0.0)
    p["warmup_frames"] = 5
    p["desired_n"] = 5
    p["filter_color_eud"] = 50.0
    p["filter_pos_eud"] = 1.0
    p["filter_norm_eud"] = 0.25
    p["filter_diff_eud"] = 0.1
    p["filter_radius"] = 5
    p["filter_diffuse"] = 0
    p["filter_sigma_spatial"] = 0.0
    p["request_id"] = 0
    p["min_trace_prob"] = 0.0
    p["bilat_color_eud"] = 1.0
    p["bilat_pos_eud"] = 1.0
    p["bilat_norm_eud"] = 1.0
    p["bilat_emit_eud"] = 0.5
    p["bilat_diff_eud"] = 0.5
    p["bilat_radius"] = 5
    p["filter_iterations"] = 1
    p["render_iterations"] = 5
    p["pt_depth_max"] = 10
    p["walk_refill"] = 0
    p["tail_from"] = -1
    p["bands"] = 0
    p["walk_ctas"] = 0
    p["carry_steps"] = 64
    p["tail_below"] = 0.0
    for k, v in over.items():
        p[k] = v
    return p


def as_params(p):
    """A PARAMS record from any record with a subset of its fields (older layouts
    included); missing fields keep their defaults."""
    out = default_params()
    if p is None:
        return out
    p = np.asarray(p)
    for name in p.dtype.names or ():
        if name in PARAMS.names:
            out[name] = p[name]
    return out


def material(diffuse=(1.0, 1.0, 1.0), emissive=(0.0, 0.0, 0.0), specular=0.5, metallic=0.0,
             roughness=0.5, transparency=0.0):
    """One RTMaterial record; texture ids -1 (untextured) as the reference default."""
    m = np.zeros((), MATERIAL)
    m["diffuse"] = diffuse
    m["emissive"] = emissive
    m["diffuseTexId"] = -1
    m["normalTexId"] = -1
    m["emissiveTexId"] = -1
    m["matType"] = 0
    m["transparency"] = transparency
    m["specular"] = specular
    m["metallic"] = metallic
    m["roughness"] = roughness
    return m
