// Cell index and in-cell offset of one coordinate as the split-precision
// mover takes them at entry.  The brick binning (particles.cu) calls the same
// function, so a particle is always binned into the brick whose records the
// tile mover stages for it: (x - xmin) / d in FP64, its floor, and an FP32
// offset that is moved to the next cell when it rounds up to 1.
#pragma once

namespace gpat {

__device__ __forceinline__ void cell_of(double x, double xmin, double d, int &c, float &f) {
    const double px = (x - xmin) / d;
    const double fl = floor(px);
    c = (int)fl;
    f = (float)(px - fl);
    if (f >= 1.0f) { f = 0.0f; c += 1; }
}

}  // namespace gpat
