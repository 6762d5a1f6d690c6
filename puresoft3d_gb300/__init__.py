"""puresoft3d_gb300: a GB300-native implementation of Puresoft3D's per-fragment
path (triangle set-up, scanline rasterisation, perspective-correct
interpolation, fragment shading, depth test, framebuffer write, 2D texture
sampling) as hand-written sm_103a CUDA behind a C ABI (include/ps3d.h)."""
