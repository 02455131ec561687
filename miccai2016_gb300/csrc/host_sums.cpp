// host_sums.cpp -- host-side sums of the sign adjustment's ridge cleaning,
// in C++ behind the C ABI (no device code).  Built with multiply-add
// contraction off, so that every product is rounded before it is added, as
// numpy rounds it, on hosts whose compilers would otherwise fuse the two.
#include <stdint.h>

#include "../../include/miccai2016_gb300.h"

// m16_segment_direction_sums: per segment the summed direction of its ridge
// points, scaled by the voxel size, that the cleaning of
// AdvancedAdjuster._do_clean_ridge (src/processing/adjust_directions.py:319-337)
// ranks segments by.  The reference sums each segment's directions over its
// points in C order of the voxels; the sums here run once over the points in
// that order, each term the double product of the float direction and the
// voxel size, added in double: the order and rounding of np.bincount with
// those products as weights.
extern "C" int m16_segment_direction_sums(const int32_t *point_label, const float *dirs3, int64_t num_points,
                                          const double *voxel_size3, int32_t num_labels, double *sums3)
{
    if (num_points < 0 || num_labels < 1 || !voxel_size3 || !sums3 ||
        (num_points > 0 && (!point_label || !dirs3)))
        return M16_ERR_BAD_ARG;
    for (int32_t l = 0; l < num_labels; ++l) sums3[3 * l] = sums3[3 * l + 1] = sums3[3 * l + 2] = 0.0;
    const double v0 = voxel_size3[0], v1 = voxel_size3[1], v2 = voxel_size3[2];
    for (int64_t i = 0; i < num_points; ++i) {
        const int32_t l = point_label[i];
        if (l < 0 || l >= num_labels) return M16_ERR_BAD_ARG;
        const double p0 = (double)dirs3[3 * i] * v0;
        const double p1 = (double)dirs3[3 * i + 1] * v1;
        const double p2 = (double)dirs3[3 * i + 2] * v2;
        sums3[3 * l] += p0;
        sums3[3 * l + 1] += p1;
        sums3[3 * l + 2] += p2;
    }
    return M16_OK;
}
