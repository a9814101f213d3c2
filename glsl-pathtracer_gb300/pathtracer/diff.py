"""Differentiable parameters of a scene, in the order pt_render_adjoint
returns their gradients: 11 per material, then 3 per light.

Per material, the raw GLSLPT::Material values (src/core/Material.h:47-119):
baseColor r, g, b, metallic, roughness, subsurface, specularTint, sheen,
sheenTint, clearcoat, clearcoatGloss; per light, emission r, g, b
(GLSLPT::Light, src/core/Scene.h:50-59).
"""
from __future__ import annotations

import numpy as np

MATERIAL_PARAMS = ("base_r", "base_g", "base_b", "metallic", "roughness", "subsurface", "specular_tint", "sheen",
                   "sheen_tint", "clearcoat", "clearcoat_gloss")
# float offsets of those values in the 32-float material record
MATERIAL_OFFSETS = np.array([0, 1, 2, 8, 9, 10, 11, 12, 13, 14, 15])
LIGHT_OFFSETS = np.array([3, 4, 5])  # emission in the 15-float light record
# valid ranges (the BSDF's domain): colours and weights in [0, 1]
LOWER, UPPER = 0.0, 1.0


def num_params(materials: np.ndarray, lights: np.ndarray) -> int:
    return materials.shape[0] * len(MATERIAL_OFFSETS) + lights.shape[0] * len(LIGHT_OFFSETS)


def get_params(materials: np.ndarray, lights: np.ndarray) -> np.ndarray:
    """Flat parameter vector (float64) of the material and light records."""
    m = np.asarray(materials, np.float64)[:, MATERIAL_OFFSETS].ravel()
    e = np.asarray(lights, np.float64)[:, LIGHT_OFFSETS].ravel()
    return np.concatenate([m, e])


def set_params(materials: np.ndarray, lights: np.ndarray, theta: np.ndarray) -> tuple[np.ndarray, np.ndarray]:
    """Copies of the records with the parameter values of theta."""
    mats = np.array(materials, np.float32, copy=True)
    lts = np.array(lights, np.float32, copy=True)
    nm = mats.shape[0] * len(MATERIAL_OFFSETS)
    mats[:, MATERIAL_OFFSETS] = np.asarray(theta[:nm], np.float32).reshape(mats.shape[0], -1)
    lts[:, LIGHT_OFFSETS] = np.asarray(theta[nm:], np.float32).reshape(lts.shape[0], -1)
    return mats, lts


def is_light_param(index: int, num_materials: int) -> bool:
    return index >= num_materials * len(MATERIAL_OFFSETS)


def perturb(theta: np.ndarray, num_materials: int, sigma: float = 0.1, seed: int = 4) -> np.ndarray:
    """theta + N(0, sigma) clamped to the valid ranges: material values to
    [0, 1], light emissions relative (x (1 + N)) and non-negative."""
    rng = np.random.RandomState(seed)
    out = np.array(theta, np.float64, copy=True)
    nm = num_materials * len(MATERIAL_OFFSETS)
    out[:nm] = np.clip(out[:nm] + rng.normal(0.0, sigma, nm), LOWER, UPPER)
    out[nm:] = np.maximum(out[nm:] * (1.0 + rng.normal(0.0, sigma, out.shape[0] - nm)), 0.0)
    return out
