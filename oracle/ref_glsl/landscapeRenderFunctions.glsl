// Stand-in for terrainwatersim/shader/landscapeRenderFunctions.glsl when the
// reference's waterRender.vert is compiled as C++ (TEST INFRASTRUCTURE).  The
// vertex shader calls one item of that file, RelPatchPosToWorldPos, which
// places a clipmap patch vertex in the world and returns its heightmap
// coordinate; here the harness chooses that coordinate directly (a texel
// centre), so that the shader's own lines after the call run on every texel.
// Found before the reference's file by the include search order.
vec2 glsl_vertex_heightmap_coord;
inline vec2 RelPatchPosToWorldPos(vec2, vec2, float, uint, vec2& heightmapCoord) {
  heightmapCoord = glsl_vertex_heightmap_coord;
  return vec2(0.0f, 0.0f);
}
