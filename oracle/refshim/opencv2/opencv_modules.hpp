// ORACLE (test infrastructure only): no optional OpenCV module is available in this stand-in.
#pragma once
