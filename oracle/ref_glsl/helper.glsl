// Stand-in for terrainwatersim/shader/helper.glsl when the reference's
// waterBrush.comp is compiled as C++ (TEST INFRASTRUCTURE).  The brush shader
// uses one item of that file, the `saturate` macro (helper.glsl:68), a clamp to
// [0, 1]; the rest of the file is rendering code that needs a graphics
// pipeline.  Found before the reference's file by the include search order.
#define saturate(value) clamp((value), 0, 1)
