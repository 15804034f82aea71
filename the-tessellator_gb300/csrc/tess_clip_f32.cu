// tess_clip_f32.cu -- FP32 instantiations of the clipping kernel (the
// FP32 + FP64-guard form); kernel source in tess_clip_impl.cuh.
#include "tess_clip_impl.cuh"

namespace tess {

cudaError_t launch_clip_f32(const ClipParams& p, int slots, int wpb, int blocks, cudaStream_t s) {
    using namespace clipk;
    const bool geo = p.geo != nullptr;
    if (slots <= 2) return geo ? launch_t<float, 2, true>(p, wpb, blocks, s) : launch_t<float, 2, false>(p, wpb, blocks, s);
    if (slots <= 4) return geo ? launch_t<float, 4, true>(p, wpb, blocks, s) : launch_t<float, 4, false>(p, wpb, blocks, s);
    return geo ? launch_t<float, 8, true>(p, wpb, blocks, s) : launch_t<float, 8, false>(p, wpb, blocks, s);
}

int clip_blocks_f32(int slots, int wpb, int device) {
    using namespace clipk;
    if (slots <= 2) return blocks_t<float, 2, false>(wpb, device);
    if (slots <= 4) return blocks_t<float, 4, false>(wpb, device);
    return blocks_t<float, 8, false>(wpb, device);
}

}  // namespace tess
