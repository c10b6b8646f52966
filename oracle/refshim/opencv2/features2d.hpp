// ORACLE (test infrastructure only): stand-in for the OpenCV features2d declarations that the
// reference's LBSP class header names. Only LBSP's static helpers are used on the background
// subtraction path; no descriptor-extractor object is ever built, so the virtual interface is
// declared and never defined.
#pragma once
#include "opencv2/core.hpp"
namespace cv {
struct KeyPoint {
    Point2f pt;
    float size = 0, angle = -1, response = 0;
    int octave = 0, class_id = -1;
};
class Feature2D : public virtual Algorithm {
public:
    virtual ~Feature2D() {}
    virtual void detect(InputArray image, std::vector<KeyPoint>& keypoints, InputArray mask = noArray());
    virtual void compute(InputArray image, std::vector<KeyPoint>& keypoints, OutputArray descriptors);
    virtual void detectAndCompute(InputArray image, InputArray mask, std::vector<KeyPoint>& keypoints,
                                  OutputArray descriptors, bool useProvidedKeypoints = false);
    virtual int descriptorSize() const;
    virtual int descriptorType() const;
    virtual int defaultNorm() const;
    virtual void write(FileStorage&) const;
    virtual void read(const FileNode&);
    virtual bool empty() const;
};
typedef Feature2D DescriptorExtractor;
}  // namespace cv
