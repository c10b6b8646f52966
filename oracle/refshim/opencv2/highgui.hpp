// ORACLE (test infrastructure only): the reference's path calls highgui only in debug-display code
// that is compiled out here; these declarations have no definitions.
#pragma once
#include "opencv2/core.hpp"
namespace cv {
void imshow(const std::string& name, InputArray img);
bool imwrite(const std::string& name, InputArray img);
int waitKey(int delay = 0);
}  // namespace cv
