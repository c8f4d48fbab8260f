"""Scene description handed to the packer: the parts of Verion's scene IR (crates/verion-scene) that
the path-tracing tables are made from.

Field names, defaults and conventions follow the reference:
`BaseBsdf` crates/verion-scene/src/material.rs:14-80, `Light` scene.rs:39-66, `Camera` scene.rs:70-94,
`LightExtra` scene.rs:178-193, `StylizationWorld` scene.rs:158-176, instance light/emit masks
scene.rs:388-420 (all ones by default).
"""
from __future__ import annotations

from dataclasses import dataclass, field
from typing import Optional, Union

import numpy as np

IDENTITY = ((1.0, 0.0, 0.0, 0.0), (0.0, 1.0, 0.0, 0.0), (0.0, 0.0, 1.0, 0.0))
ALL = 0xFFFFFFFF


@dataclass
class Mesh:
    positions: np.ndarray            # (n, 3) float32
    indices: np.ndarray              # (3 m,) uint32
    normals: Optional[np.ndarray] = None  # (n, 3) float32
    uvs: Optional[np.ndarray] = None      # (n, 2) float32

    def __post_init__(self):
        self.positions = np.ascontiguousarray(self.positions, dtype=np.float32).reshape(-1, 3)
        self.indices = np.ascontiguousarray(self.indices, dtype=np.uint32).reshape(-1)
        if self.indices.size % 3:
            raise ValueError("index count is not a multiple of 3")
        if self.indices.size and int(self.indices.max()) >= len(self.positions):
            raise ValueError("index beyond the vertex count")
        if self.normals is not None:
            self.normals = np.ascontiguousarray(self.normals, dtype=np.float32).reshape(-1, 3)
        if self.uvs is not None:
            self.uvs = np.ascontiguousarray(self.uvs, dtype=np.float32).reshape(-1, 2)


@dataclass
class Image:
    width: int
    height: int
    pixels: np.ndarray  # (height * width, 3) float32, row-major from the top

    def __post_init__(self):
        self.pixels = np.ascontiguousarray(self.pixels, dtype=np.float32).reshape(-1, 3)
        if len(self.pixels) != self.width * self.height or self.width == 0 or self.height == 0:
            raise ValueError("image size does not match its pixels")


@dataclass
class BaseBsdf:
    base_color: tuple = (0.8, 0.8, 0.8)
    metallic: float = 0.0
    roughness: float = 0.5
    transmission: float = 0.0
    ior: float = 1.5
    clearcoat: float = 0.0
    clearcoat_roughness: float = 0.0
    sheen_color: tuple = (0.0, 0.0, 0.0)
    sheen_roughness: float = 0.0
    dispersion: float = 0.0
    opacity: float = 1.0
    opacity_texture: Optional[int] = None
    emission: tuple = (0.0, 0.0, 0.0)
    base_color_texture: Optional[int] = None
    metallic_roughness_texture: Optional[int] = None
    emission_texture: Optional[int] = None
    normal_texture: Optional[int] = None
    normal_scale: float = 1.0


@dataclass
class Instance:
    mesh: int
    material: int
    transform: tuple = IDENTITY  # 3x4 row-major object-to-world


@dataclass
class Point:
    position: tuple
    color: tuple
    intensity: float


@dataclass
class Directional:
    direction: tuple  # the direction the light travels
    color: tuple
    intensity: float


@dataclass
class Spot:
    position: tuple
    direction: tuple
    color: tuple
    intensity: float
    inner_cone: float
    outer_cone: float


@dataclass
class Environment:
    color: tuple


@dataclass
class EnvironmentMap:
    image: int
    scale: float = 1.0


Light = Union[Point, Directional, Spot, Environment, EnvironmentMap]


@dataclass
class IesProfile:
    """361 horizontal rows of 181 vertical samples at one degree (crates/verion-scene/src/ies.rs)."""
    table: np.ndarray

    def __post_init__(self):
        self.table = np.ascontiguousarray(self.table, dtype=np.float32).reshape(-1)
        if self.table.size != 361 * 181:
            raise ValueError("an IES table has 361 x 181 samples")


@dataclass
class LightExtra:
    link_mask: int = ALL
    ies: Optional[tuple] = None  # (IesProfile, 3x3 world frame rows x, y, z)


@dataclass
class Camera:
    transform: tuple = IDENTITY  # camera-to-world, looking down -z
    vertical_fov: float = 0.8
    focus_distance: float = 1.0
    aperture_radius: float = 0.0
    shift: tuple = (0.0, 0.0)


@dataclass
class StylizationWorld:
    virtual_light: bool = True
    direction: Optional[tuple] = None
    strength: float = 1.0


@dataclass
class Scene:
    meshes: list = field(default_factory=list)
    materials: list = field(default_factory=list)
    instances: list = field(default_factory=list)
    lights: list = field(default_factory=list)
    images: list = field(default_factory=list)
    camera: Camera = field(default_factory=Camera)
    light_extras: dict = field(default_factory=dict)    # light index -> LightExtra
    instance_masks: dict = field(default_factory=dict)  # instance index -> receive mask
    emit_masks: dict = field(default_factory=dict)      # instance index -> emit group mask
    stylization_world: StylizationWorld = field(default_factory=StylizationWorld)
    transparent_background: bool = False

    def add_mesh(self, mesh: Mesh) -> int:
        self.meshes.append(mesh)
        return len(self.meshes) - 1

    def add_material(self, m: BaseBsdf) -> int:
        self.materials.append(m)
        return len(self.materials) - 1

    def add_instance(self, inst: Instance) -> int:
        if not (0 <= inst.mesh < len(self.meshes)) or not (0 <= inst.material < len(self.materials)):
            raise ValueError("instance refers to a missing mesh or material")
        self.instances.append(inst)
        return len(self.instances) - 1

    def add_light(self, light, extra: Optional[LightExtra] = None) -> int:
        self.lights.append(light)
        if extra is not None:
            self.light_extras[len(self.lights) - 1] = extra
        return len(self.lights) - 1

    def add_image(self, image: Image) -> int:
        self.images.append(image)
        return len(self.images) - 1

    def instance_light_mask(self, i: int) -> int:
        return self.instance_masks.get(i, ALL)

    def instance_emit_mask(self, i: int) -> int:
        return self.emit_masks.get(i, ALL)

    def light_extra(self, i: int) -> LightExtra:
        return self.light_extras.get(i, LightExtra())
