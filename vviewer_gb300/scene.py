"""Scene model mirroring vengine's core scene API, flattened into the buffers
the path tracer reads.

Names and defaults follow the reference:
  Transform            src/lib/vengine/math/Transform.cpp:8-115 (model = T * R(quat) * S)
  PerspectiveCamera    src/lib/vengine/core/Camera.hpp:14-104, Camera.cpp:38-41 (lookAt, forward = -Z)
  Materials            src/lib/vengine/vulkan/resources/VulkanMaterial.cpp:30-62 (PBR), :225-250 (Lambert),
                       :438-483 (volume packing)
  Lights               src/lib/vengine/core/Light.hpp:16-98, VulkanScene.cpp:115-142 (colour (1,1,1,1))
  Scene / SceneData    src/lib/vengine/core/Scene.cpp:31-44, 147-159
  InstancesManager     src/lib/vengine/core/Instances.cpp:76-181 (slot order: opaque mesh groups,
                       transparent objects, light objects)
  Light instances      src/lib/vengine/vulkan/VulkanInstances.cpp:66-109
  render() set-up      src/lib/vengine/vulkan/renderers/VulkanRendererPathTracing.cpp:143-199
"""
from __future__ import annotations

import ctypes as C
import enum
import math
from dataclasses import dataclass, field

import numpy as np

from . import _native as N

f32 = np.float32


# ---------------------------------------------------------------- math (glm conventions, float32)

def radians(deg: float) -> float:
    return float(f32(deg) * f32(math.pi / 180.0))


def quat_from_euler(e) -> np.ndarray:
    """glm::quat(vec3 eulerAngles): (w, x, y, z)."""
    e = np.asarray(e, dtype=f32) * f32(0.5)
    c = np.cos(e).astype(f32)
    s = np.sin(e).astype(f32)
    w = c[0] * c[1] * c[2] + s[0] * s[1] * s[2]
    x = s[0] * c[1] * c[2] - c[0] * s[1] * s[2]
    y = c[0] * s[1] * c[2] + s[0] * c[1] * s[2]
    z = c[0] * c[1] * s[2] - s[0] * s[1] * c[2]
    return np.array([w, x, y, z], dtype=f32)


def quat_to_mat3(q) -> np.ndarray:
    """glm::mat3_cast as a row-major matrix."""
    w, x, y, z = (f32(v) for v in q)
    xx, yy, zz = x * x, y * y, z * z
    xz, xy, yz = x * z, x * y, y * z
    wx, wy, wz = w * x, w * y, w * z
    one, two = f32(1), f32(2)
    return np.array([
        [one - two * (yy + zz), two * (xy - wz), two * (xz + wy)],
        [two * (xy + wz), one - two * (xx + zz), two * (yz - wx)],
        [two * (xz - wy), two * (yz + wx), one - two * (xx + yy)],
    ], dtype=f32)


def quat_rotate(q, v) -> np.ndarray:
    """glm::rotate(quat, vec3) = q * v."""
    w = f32(q[0])
    qv = np.asarray(q[1:], dtype=f32)
    v = np.asarray(v, dtype=f32)
    uv = np.cross(qv, v).astype(f32)
    uuv = np.cross(qv, uv).astype(f32)
    return (v + ((uv * w) + uuv) * f32(2)).astype(f32)


def normalize(v) -> np.ndarray:
    v = np.asarray(v, dtype=f32)
    return (v * (f32(1) / np.sqrt(np.dot(v, v)))).astype(f32)


def look_at(eye, center, up) -> np.ndarray:
    """glm::lookAt (right-handed), row-major 4x4."""
    eye = np.asarray(eye, dtype=f32)
    f = normalize(np.asarray(center, dtype=f32) - eye)
    s = normalize(np.cross(f, np.asarray(up, dtype=f32)))
    u = np.cross(s, f).astype(f32)
    m = np.eye(4, dtype=f32)
    m[0, :3] = s
    m[1, :3] = u
    m[2, :3] = -f
    m[0, 3] = -np.dot(s, eye)
    m[1, 3] = -np.dot(u, eye)
    m[2, 3] = np.dot(f, eye)
    return m


def perspective(fovy: float, aspect: float, znear: float, zfar: float) -> np.ndarray:
    """glm::perspective, right-handed, depth in [0, 1] (GLM_FORCE_DEPTH_ZERO_TO_ONE, Camera.hpp:5)."""
    t = f32(math.tan(f32(fovy) / f32(2)))
    m = np.zeros((4, 4), dtype=f32)
    m[0, 0] = f32(1) / (f32(aspect) * t)
    m[1, 1] = f32(1) / t
    m[2, 2] = f32(zfar) / (f32(znear) - f32(zfar))
    m[3, 2] = f32(-1)
    m[2, 3] = -(f32(zfar) * f32(znear)) / (f32(zfar) - f32(znear))
    return m


def inverse(m: np.ndarray) -> np.ndarray:
    return np.linalg.inv(m.astype(np.float64)).astype(f32)


def colmajor(m: np.ndarray) -> list:
    return [float(v) for v in np.asarray(m, dtype=f32).T.reshape(-1)]


# ---------------------------------------------------------------- transform / camera

class Transform:
    """Position, rotation (quaternion, or Euler angles in radians) and scale."""

    def __init__(self, position=(0, 0, 0), scale=(1, 1, 1), rotation=None):
        self.position = np.asarray(position, dtype=f32)
        self.scale = np.asarray(scale, dtype=f32)
        if rotation is None:
            self.rotation = np.array([1, 0, 0, 0], dtype=f32)
        elif len(rotation) == 3:
            self.rotation = quat_from_euler(rotation)
        else:
            self.rotation = np.asarray(rotation, dtype=f32)

    def set_rotation(self, q) -> None:
        self.rotation = quat_from_euler(q) if len(q) == 3 else np.asarray(q, dtype=f32)

    def forward(self):
        return -quat_rotate(self.rotation, (0, 0, 1))

    def up(self):
        return quat_rotate(self.rotation, (0, 1, 0))

    def model_matrix(self) -> np.ndarray:
        m = np.eye(4, dtype=f32)
        r = quat_to_mat3(self.rotation)
        m[:3, :3] = (r * self.scale[None, :]).astype(f32)
        m[:3, 3] = self.position
        return m


class PerspectiveCamera:
    def __init__(self):
        self.transform = Transform()
        self.fov = 60.0
        self.znear = 0.5
        self.zfar = 50.0
        self.lens_radius = 0.0
        self.focal_distance = 10.0
        self.volume: "MaterialVolume | None" = None

    def view_matrix(self) -> np.ndarray:
        p = self.transform.position
        return look_at(p, p + self.transform.forward(), self.transform.up())

    def projection_matrix(self, width: int, height: int) -> np.ndarray:
        m = perspective(radians(self.fov), float(f32(width) / f32(height)), self.znear, self.zfar)
        m[1, 1] *= f32(-1)
        return m


# ---------------------------------------------------------------- materials / lights / meshes

class MaterialType(enum.IntEnum):
    PBR_STANDARD = 0
    SKYBOX = 1
    LAMBERT = 2
    VOLUME = 3


TEX_WHITE, TEX_WHITE_COLOR, TEX_NORMAL_DEFAULT = 0, 1, 2


def _is_black(c, thr):
    return all(abs(float(x)) < thr for x in c)


class Material:
    type = MaterialType.PBR_STANDARD

    def __init__(self, name: str):
        self.name = name
        self.index = -1
        self.transparent = False

    def set_transparent(self, t: bool) -> None:
        self.transparent = bool(t)

    def is_emissive(self) -> bool:
        return False

    def is_transparent(self) -> bool:
        return self.transparent


class MaterialPBRStandard(Material):
    type = MaterialType.PBR_STANDARD

    def __init__(self, name: str):
        super().__init__(name)
        self.albedo = [1.0, 1.0, 1.0, 1.0]
        self.metallic = 0.0
        self.roughness = 1.0
        self.ao = 1.0
        self.emissive = [0.0, 0.0, 0.0, 1.0]
        self.u_tiling = 1.0
        self.v_tiling = 1.0
        self.albedo_texture = TEX_WHITE_COLOR
        self.metallic_texture = TEX_WHITE
        self.roughness_texture = TEX_WHITE
        self.ao_texture = TEX_WHITE
        self.emissive_texture = TEX_WHITE_COLOR
        self.normal_texture = TEX_NORMAL_DEFAULT
        self.alpha_texture = TEX_WHITE

    def emissive_color(self):
        return [self.emissive[i] * self.emissive[3] for i in range(3)]

    def is_emissive(self) -> bool:
        # Material.cpp:85-88
        return self.emissive[3] > float(np.finfo(np.float32).eps) and not _is_black(self.emissive_color(), 0.01)

    def pack(self) -> N.Material:
        m = N.Material()
        m.albedo[:] = self.albedo
        m.metallic_roughness_ao[:] = [self.metallic, self.roughness, self.ao, 1.0 if self.transparent else 0.0]
        m.emissive[:] = self.emissive
        m.textures1[:] = [self.albedo_texture, self.metallic_texture, self.roughness_texture, self.ao_texture]
        m.textures2[:] = [self.emissive_texture, self.normal_texture, 0, self.alpha_texture]
        m.uv_tiling[:] = [self.u_tiling, self.v_tiling, float(MaterialType.PBR_STANDARD), 0.0]
        return m


class MaterialLambert(Material):
    type = MaterialType.LAMBERT

    def __init__(self, name: str):
        super().__init__(name)
        self.albedo = [1.0, 1.0, 1.0, 1.0]
        self.ao = 1.0
        self.emissive = [0.0, 0.0, 0.0, 1.0]
        self.u_tiling = 1.0
        self.v_tiling = 1.0
        self.albedo_texture = TEX_WHITE_COLOR
        self.ao_texture = TEX_WHITE
        self.emissive_texture = TEX_WHITE_COLOR
        self.normal_texture = TEX_NORMAL_DEFAULT
        self.alpha_texture = TEX_WHITE

    def emissive_color(self):
        return [self.emissive[i] * self.emissive[3] for i in range(3)]

    def is_emissive(self) -> bool:
        # Material.cpp:140-143
        return self.emissive[3] > float(np.finfo(np.float32).eps) and not _is_black(self.emissive_color(), 0.01)

    def pack(self) -> N.Material:
        m = N.Material()
        m.albedo[:] = self.albedo
        m.metallic_roughness_ao[:] = [0.0, 0.0, self.ao, 1.0 if self.transparent else 0.0]
        m.emissive[:] = self.emissive
        m.textures1[:] = [self.albedo_texture, 0, 0, self.ao_texture]
        m.textures2[:] = [self.emissive_texture, self.normal_texture, 0, self.alpha_texture]
        m.uv_tiling[:] = [self.u_tiling, self.v_tiling, float(MaterialType.LAMBERT), 0.0]
        return m


class MaterialVolume(Material):
    """Homogeneous medium: sigma_a -> albedo, sigma_s -> metallicRoughnessAO, g -> emissive.r."""
    type = MaterialType.VOLUME

    def __init__(self, name: str):
        super().__init__(name)
        self.sigma_s = [0.2, 0.2, 0.2, 0.2]
        self.sigma_a = [0.01, 0.01, 0.01, 0.01]
        self.g = 0.0

    def pack(self) -> N.Material:
        m = N.Material()
        m.albedo[:] = self.sigma_a
        m.metallic_roughness_ao[:] = self.sigma_s
        m.emissive[:] = [self.g, 0.0, 0.0, 0.0]
        m.uv_tiling[:] = [1.0, 1.0, float(MaterialType.VOLUME), 0.0]
        return m


class LightType(enum.IntEnum):
    POINT_LIGHT = 0
    DIRECTIONAL_LIGHT = 1
    MESH_LIGHT = 2
    ENVIRONMENT_MAP = 3


class Light:
    type = LightType.POINT_LIGHT

    def __init__(self, name: str, color=(1.0, 1.0, 1.0, 1.0)):
        self.name = name
        self.color = list(color)
        self.index = -1


class PointLight(Light):
    type = LightType.POINT_LIGHT


class DirectionalLight(Light):
    type = LightType.DIRECTIONAL_LIGHT


@dataclass
class Mesh:
    """Vertex array (numpy structured, vvpt_vertex layout) and triangle indices (N x 3 uint32)."""
    name: str
    vertices: np.ndarray
    indices: np.ndarray
    index: int = -1

    @property
    def num_triangles(self) -> int:
        return int(self.indices.shape[0])


VERTEX_DTYPE = np.dtype([("position", f32, 3), ("uv", f32, 2), ("normal", f32, 3), ("color", f32, 3),
                         ("tangent", f32, 3), ("bitangent", f32, 3)])
assert VERTEX_DTYPE.itemsize == C.sizeof(N.Vertex)


class EnvironmentType(enum.IntEnum):
    SOLID_COLOR = 0
    HDRI = 1
    SOLID_COLOR_WITH_HDRI_LIGHTING = 2


# ---------------------------------------------------------------- scene graph

class SceneObject:
    _next_id = 1

    def __init__(self, scene: "Scene", name: str, transform: Transform):
        self.scene = scene
        self.name = name
        self.local_transform = transform
        self.children: list[SceneObject] = []
        self.parent: SceneObject | None = None
        self.mesh: Mesh | None = None
        self.material: Material | None = None
        self.light: Light | None = None
        self.cast_shadows = True
        self.volume_front: MaterialVolume | None = None
        self.volume_back: MaterialVolume | None = None
        self.active = True
        self.id = SceneObject._next_id
        SceneObject._next_id += 1

    def set_local_transform(self, t: Transform) -> None:
        self.local_transform = t

    def model_matrix(self) -> np.ndarray:
        m = self.local_transform.model_matrix()
        if self.parent is not None:
            m = (self.parent.model_matrix().astype(f32) @ m).astype(f32)
        return m

    def world_position(self):
        return self.model_matrix()[:3, 3]

    def flat(self) -> list["SceneObject"]:
        out = []
        for c in self.children:
            out.append(c)
            out.extend(c.flat())
        return out


class Scene:
    def __init__(self, engine: "Engine"):
        self.engine = engine
        self.camera = PerspectiveCamera()
        self.roots: list[SceneObject] = []
        self.environment_type = EnvironmentType.SOLID_COLOR
        self.background_color = [0.0, 0.0, 0.0]
        self.environment_intensity = 1.0
        self.exposure = 0.0
        self.environment_map: np.ndarray | None = None  # H x W x 4 float32 equirect

    def add_scene_object(self, name: str, transform: Transform | None = None,
                         parent: SceneObject | None = None) -> SceneObject:
        so = SceneObject(self, name, transform or Transform())
        if parent is None:
            self.roots.append(so)
        else:
            so.parent = parent
            parent.children.append(so)
        return so

    def clear(self) -> None:
        """Removes the objects only (camera, environment and background stay,
        as Scene::clear, src/lib/vengine/core/Scene.cpp:184-205)."""
        self.roots = []

    def objects_flat(self) -> list[SceneObject]:
        out = []
        for r in self.roots:
            out.append(r)
            out.extend(r.flat())
        return out

    # -------------------------------------------------- flattening

    def build(self) -> "FlatScene":
        """InstancesManager::build + VulkanInstancesManager::build."""
        opaque: dict[int, list[SceneObject]] = {}
        opaque_mesh: dict[int, Mesh] = {}
        transparent: list[SceneObject] = []
        lights: list[SceneObject] = []
        mesh_lights: list[SceneObject] = []
        volumes: list[SceneObject] = []
        for so in self.objects_flat():
            if not so.active:
                continue
            if so.mesh is not None and so.material is not None:
                if so.material.is_emissive():
                    mesh_lights.append(so)
                if not so.material.is_transparent():
                    key = id(so.mesh)
                    opaque.setdefault(key, []).append(so)
                    opaque_mesh[key] = so.mesh
                else:
                    transparent.append(so)
            if so.light is not None:
                lights.append(so)
            if so.volume_front is not None or so.volume_back is not None:
                volumes.append(so)

        slots: list[tuple[SceneObject, bool]] = []  # (object, in TLAS)
        for key, objs in opaque.items():
            for so in objs:
                slots.append((so, True))
        for so in transparent:
            slots.append((so, True))
        for so in lights:
            slots.append((so, False))
        first_slot: dict[int, int] = {}
        for i, (so, _) in enumerate(slots):
            first_slot.setdefault(id(so), i)

        fs = FlatScene()
        fs.meshes = self.engine.meshes
        for so, in_tlas in slots:
            inst = N.Instance()
            inst.model[:] = colmajor(so.model_matrix())
            idv = [float(so.id), -1.0, -1.0, 0.0]
            if so.volume_front is not None:
                idv[1] = float(so.volume_front.index)
            if so.volume_back is not None:
                idv[2] = float(so.volume_back.index)
            inst.id[:] = idv
            inst.material_index = so.material.index if so.material is not None else 0
            if so.mesh is not None:
                inst.mesh_index = so.mesh.index
                inst.num_triangles = so.mesh.num_triangles
            else:
                inst.mesh_index = 0xFFFFFFFF
                inst.num_triangles = 0
            inst.flags = N.INSTANCE_IN_TLAS if in_tlas else 0
            fs.instances.append(inst)

        for so in lights:
            li = N.LightInstance()
            light = so.light
            li.info[0] = light.index
            li.info[1] = first_slot[id(so)]
            li.info[3] = int(light.type)
            m = so.model_matrix()
            if light.type == LightType.POINT_LIGHT:
                p = so.world_position()
                li.position[:] = [float(p[0]), float(p[1]), float(p[2]), 1.0 if so.cast_shadows else 0.0]
            elif light.type == LightType.DIRECTIONAL_LIGHT:
                d = (m @ np.array([0, 0, 1, 0], dtype=f32)).astype(f32)
                li.position[:] = [float(d[0]), float(d[1]), float(d[2]), 1.0 if so.cast_shadows else 0.0]
            fs.lights.append(li)
        for so in mesh_lights:
            li = N.LightInstance()
            li.info[1] = first_slot[id(so)]
            li.info[3] = int(LightType.MESH_LIGHT)
            m = so.model_matrix()
            li.position[:] = [float(v) for v in m[0, :]]
            li.position1[:] = [float(v) for v in m[1, :]]
            li.position2[:] = [float(v) for v in m[2, :]]
            fs.lights.append(li)

        fs.materials = [m.pack() for m in self.engine.materials]
        fs.light_data = []
        for light in self.engine.lights:
            ld = N.LightData()
            ld.color[:] = light.color
            ld.type[0] = int(light.type)
            fs.light_data.append(ld)
        fs.textures = self.engine.textures
        fs.environment = self.environment_map
        fs.volumes = volumes
        return fs

    def scene_data(self, width: int, height: int) -> N.SceneData:
        """SceneData for a render at width x height (VulkanRendererPathTracing.cpp:143-194)."""
        cam = self.camera
        sd = N.SceneData()
        view = cam.view_matrix()
        proj = cam.projection_matrix(width, height)
        sd.view[:] = colmajor(view)
        sd.view_inverse[:] = colmajor(inverse(view))
        sd.projection[:] = colmajor(proj)
        sd.projection_inverse[:] = colmajor(inverse(proj))
        sd.exposure[:] = [self.exposure, self.environment_intensity, cam.lens_radius, cam.focal_distance]
        sd.background[:] = [*self.background_color[:3], float(int(self.environment_type))]
        vol = -1.0
        if cam.volume is not None and cam.volume.type == MaterialType.VOLUME:
            vol = float(cam.volume.index)
        sd.volumes[:] = [vol, cam.znear, cam.zfar, 0.0]
        return sd


class FlatScene:
    """The reference's GPU-side buffers for one scene, ready for vvpt_scene_upload."""

    def __init__(self):
        self.meshes: list[Mesh] = []
        self.instances: list[N.Instance] = []
        self.materials: list[N.Material] = []
        self.light_data: list[N.LightData] = []
        self.lights: list[N.LightInstance] = []
        self.textures: list[tuple[int, np.ndarray]] = []
        self.environment: np.ndarray | None = None
        self._keep: list = []

    @property
    def num_lights(self) -> int:
        return len(self.lights)

    def desc(self) -> N.SceneDesc:
        keep = []

        def arr(ctype, items):
            a = (ctype * max(1, len(items)))(*items)
            keep.append(a)
            return a

        mdescs = []
        for m in self.meshes:
            v = np.ascontiguousarray(m.vertices)
            ix = np.ascontiguousarray(m.indices, dtype=np.uint32)
            keep.extend([v, ix])
            mdescs.append(N.MeshDesc(v.ctypes.data, len(v), ix.ctypes.data, ix.shape[0]))
        tdescs = []
        for fmt, img in self.textures:
            img = np.ascontiguousarray(img)
            keep.append(img)
            tdescs.append(N.TextureDesc(img.shape[1], img.shape[0], fmt, 0, img.ctypes.data))
        d = N.SceneDesc()
        d.meshes = arr(N.MeshDesc, mdescs)
        d.num_meshes = len(mdescs)
        d.instances = arr(N.Instance, self.instances)
        d.num_instances = len(self.instances)
        d.materials = arr(N.Material, self.materials)
        d.num_materials = len(self.materials)
        d.light_data = arr(N.LightData, self.light_data)
        d.num_light_data = len(self.light_data)
        d.lights = arr(N.LightInstance, self.lights)
        d.num_lights = len(self.lights)
        d.textures = arr(N.TextureDesc, tdescs)
        d.num_textures = len(tdescs)
        if self.environment is not None:
            env = np.ascontiguousarray(self.environment, dtype=f32)
            keep.append(env)
            td = N.TextureDesc(env.shape[1], env.shape[0], N.TEXTURE_RGBA32F, 0, env.ctypes.data)
            keep.append(td)
            d.environment = C.pointer(td)
        self._keep = keep
        return d


# ---------------------------------------------------------------- engine (asset registries)

def default_textures() -> list[tuple[int, np.ndarray]]:
    """white (linear), whiteColor (sRGB), normalmapdefault (0x80, 0x80, 0xFF):
    src/lib/vengine/vulkan/resources/VulkanTextures.cpp:73-75, src/lib/vengine/core/Image.hpp:40-88."""
    white = np.full((1, 1, 4), 255, dtype=np.uint8)
    normal = np.array([[[0x80, 0x80, 0xFF, 0xFF]]], dtype=np.uint8)
    return [(N.TEXTURE_RGBA8_LINEAR, white), (N.TEXTURE_RGBA8_SRGB, white.copy()), (N.TEXTURE_RGBA8_LINEAR, normal)]


class Engine:
    """Asset registries (materials, lights, meshes, textures) plus one scene.

    Material and light indices are creation order, as the reference's UBO
    blocks. The engine's default assets are created first
    (src/lib/vengine/vulkan/VulkanEngine.cpp:331-376)."""

    def __init__(self, with_defaults: bool = True):
        self.materials: list[Material] = []
        self.lights: list[Light] = []
        self.meshes: list[Mesh] = []
        self.textures = default_textures()
        self.models: dict = {}  # imported models by name (model3d.import_model)
        self._materials_by_name: dict[str, Material] = {}
        self._lights_by_name: dict[str, Light] = {}
        self.scene = Scene(self)
        if with_defaults:
            m = self.create_material(MaterialPBRStandard, "defaultMaterial")
            m.albedo = [0.8, 0.8, 0.8, 1.0]
            m.metallic = 0.5
            m.roughness = 0.5
            m.ao = 1.0
            m.emissive = [0.0, 0.0, 0.0, 1.0]
            e = self.create_material(MaterialPBRStandard, "defaultEmissive")
            e.albedo = [1.0, 1.0, 1.0, 1.0]
            e.emissive = [1.0, 1.0, 1.0, 1.0]
            v = self.create_material(MaterialVolume, "defaultVolume")
            v.sigma_s = [0.01, 0.01, 0.01, 1.0]
            v.sigma_a = [0.01, 0.01, 0.01, 1.0]
            v.g = 0.0
            self.create_light("defaultPointLight", LightType.POINT_LIGHT).color = [1.0, 1.0, 1.0, 1.0]
            self.create_light("defaultDirectionalLightSun", LightType.DIRECTIONAL_LIGHT).color = [1.0, 0.9, 0.8, 1.0]
            self.create_light("defaultDirectionalLightMoon", LightType.DIRECTIONAL_LIGHT).color = [0.31, 0.4, 0.52, 1.0]

    def create_material(self, cls, name: str):
        if name in self._materials_by_name:
            return self._materials_by_name[name]
        m = cls(name)
        m.index = len(self.materials)
        self.materials.append(m)
        self._materials_by_name[name] = m
        return m

    def material(self, name: str) -> Material:
        return self._materials_by_name[name]

    def create_light(self, name: str, type_: LightType, color=(1.0, 1.0, 1.0, 1.0)) -> Light:
        """VulkanScene::createLight: returns the existing light of that name."""
        if name in self._lights_by_name:
            return self._lights_by_name[name]
        cls = PointLight if type_ == LightType.POINT_LIGHT else DirectionalLight
        light = cls(name, color)
        light.index = len(self.lights)
        self.lights.append(light)
        self._lights_by_name[name] = light
        return light

    def light(self, name: str) -> Light:
        return self._lights_by_name[name]

    def add_mesh(self, mesh: Mesh) -> Mesh:
        mesh.index = len(self.meshes)
        self.meshes.append(mesh)
        return mesh

    def add_texture(self, fmt: int, image: np.ndarray) -> int:
        self.textures.append((fmt, image))
        return len(self.textures) - 1
