// ORACLE (test infrastructure only): stand-in for cv::BackgroundSubtractor, the interface the
// reference's IIBackgroundSubtractor derives from (BackgroundSubtractionUtils.hpp:24).
#pragma once
#include "opencv2/core.hpp"
namespace cv {
class BackgroundSubtractor : public Algorithm {
public:
    virtual ~BackgroundSubtractor() {}
    virtual void apply(InputArray image, OutputArray fgmask, double learningRate = -1) = 0;
    virtual void getBackgroundImage(OutputArray backgroundImage) const = 0;
};
}  // namespace cv
