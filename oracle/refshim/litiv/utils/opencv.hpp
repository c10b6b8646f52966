// ORACLE (test infrastructure only): slim replacement for the reference's litiv/utils/opencv.hpp.
// The full header needs most of OpenCV (display helpers, allocators, sparse matrices, archives);
// the background subtraction path uses only its pixel sampling helpers, so this header provides
// the OpenCV stand-ins and includes the reference's own helpers (clampImageCoords,
// getSamplePosition, getSamplePosition_3x3_std1/_7x7_std2, getNeighborPosition,
// getNeighborPosition_3x3/_5x5; modules/utils/include/litiv/utils/opencv.hpp), cut out unmodified
// by oracle/refshim/build_ref.py into lv_sampling_helpers.inc.
#pragma once

#include "litiv/utils/simd.hpp"
#include <opencv2/core.hpp>
#include <opencv2/imgproc.hpp>
#include <opencv2/highgui.hpp>

namespace lv {

struct MatInfo;

// cv-compatible scalar element types (declared for the reference's math.hpp templates)
template <typename TData>
constexpr bool isDataTypeCompat() {
    return std::is_same<TData, uchar>::value || std::is_same<TData, schar>::value ||
           std::is_same<TData, ushort>::value || std::is_same<TData, short>::value ||
           std::is_same<TData, int>::value || std::is_same<TData, float>::value || std::is_same<TData, double>::value;
}

// the debug display helper of IIParallelAlgo (algo.hpp); never created here
struct DisplayHelper {
    cv::FileStorage m_oFS;
    std::string m_sDisplayName;
};
using DisplayHelperPtr = std::shared_ptr<DisplayHelper>;

#include "lv_sampling_helpers.inc"

}  // namespace lv
