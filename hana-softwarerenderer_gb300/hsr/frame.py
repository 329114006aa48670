"""One DrawModel::draw (scene.h:53-99) on the GPU through the C ABI.

The shadow pass renders the mesh with ShadowShader into the shadow target, the main pass
reads it as ShaderData::shadow_map; both clears (main.cpp:152-153 for the frame buffer,
scene.h:94-98 for the shadow map) are fused into the draws, so every pixel is written
once per frame.
"""
from __future__ import annotations

from . import DrawDesc, Mesh, Target, Texture, draw, draw_batch, make_desc
from . import scenes


class GpuFrame:
    def __init__(self, frame: "scenes.Frame", mesh: Mesh | None = None):
        self.frame = frame
        self.mesh = mesh or Mesh(frame.mesh)
        self._own_mesh = mesh is None
        self.diffuse = Texture(frame.diffuse) if frame.diffuse is not None else None
        self.normal = Texture(frame.normal) if frame.normal is not None else None
        self.main = Target(frame.width, frame.height)
        sw, sh = frame.shadow_size
        self.shadow = Target(sw, sh) if sw > 0 else None
        self._keep: list = []
        self.descs: list[DrawDesc] = []
        if self.shadow is not None:
            self.descs.append(make_desc(self.mesh, scenes.SHADOW, frame.sd, self.shadow, self.diffuse, self.normal,
                                        clear=(frame.shadow_clear_rgba, frame.shadow_clear_depth), keep=self._keep))
        self.descs.append(make_desc(self.mesh, frame.shader, frame.sd, self.main, self.diffuse, self.normal,
                                    shadow_map=self.shadow, clear=(frame.clear_rgba, frame.clear_depth),
                                    keep=self._keep))

    def render(self, batched: bool = True) -> None:
        if batched:
            draw_batch(self.descs)
        else:
            for d in self.descs:
                draw(d)

    def download(self) -> dict:
        out = {"main": self.main.download()}
        if self.shadow is not None:
            out["shadow"] = self.shadow.download()
        return out

    def release(self) -> None:
        for obj in (self.main, self.shadow, self.diffuse, self.normal):
            if obj is not None:
                obj.release()
        if self._own_mesh:
            self.mesh.release()
