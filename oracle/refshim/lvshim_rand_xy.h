/* ORACLE (test infrastructure only): force-included after lvshim_rand.h for
 * modules/video/src/BackgroundSubtractorViBe.cpp and BackgroundSubtractorPBAS.cpp alone. Their pixel loops
 * declare no nPxIter: they name the pixel (x, y) (ViBe's initialize(): (x_orig, y_orig)). The namespace-scope sentinels below
 * carry those names, so inside a loop the loop variables shadow them and rand() is attributed to the
 * loop's pixel (the same keying as the other algorithms: draw k of pixel p in frame t). */
#ifndef LV_ORACLE_SHIM_RAND_XY_H
#define LV_ORACLE_SHIM_RAND_XY_H
#undef rand
static const int x = -1, y = -1, x_orig = -1, y_orig = -1;
int lvshim_rand_xy(int px, int py, int px_orig, int py_orig, int width);
#define rand() lvshim_rand_xy(x, y, x_orig, y_orig, m_oImgSize.width)
#endif
