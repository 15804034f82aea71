// tess_clip_f64.cu -- FP64 instantiations of the clipping kernel (the
// plain FP64 form and the FP64 re-runs); kernel source in tess_clip_impl.cuh.
#include "tess_clip_impl.cuh"

namespace tess {

cudaError_t launch_clip_f64(const ClipParams& p, int slots, int form, int wpb, int blocks, cudaStream_t s) {
    using namespace clipk;
    const bool geo = p.geo != nullptr;
    if (slots <= 2) {
        if (geo) return launch_t<double, 2, true, kFormStd>(p, wpb, blocks, s);
        return form == kFormLean ? launch_t<double, 2, false, kFormLean>(p, wpb, blocks, s)
                                 : launch_t<double, 2, false, kFormStd>(p, wpb, blocks, s);
    }
    if (slots <= 4)
        return geo ? launch_t<double, 4, true, kFormStd>(p, wpb, blocks, s) : launch_t<double, 4, false, kFormStd>(p, wpb, blocks, s);
    return geo ? launch_t<double, 8, true, kFormStd>(p, wpb, blocks, s) : launch_t<double, 8, false, kFormStd>(p, wpb, blocks, s);
}

int clip_blocks_f64(int slots, int form, int wpb, int device) {
    using namespace clipk;
    if (slots <= 2) {
        return form == kFormLean ? blocks_t<double, 2, false, kFormLean>(wpb, device)
                                 : blocks_t<double, 2, false, kFormStd>(wpb, device);
    }
    if (slots <= 4) return blocks_t<double, 4, false, kFormStd>(wpb, device);
    return blocks_t<double, 8, false, kFormStd>(wpb, device);
}

}  // namespace tess
