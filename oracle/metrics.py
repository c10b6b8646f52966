"""ORACLE (test infrastructure only): restatement of the reference's change-detection evaluation.

lv::BinClassif::accumulate (modules/datasets/src/metrics.cpp:21-61) and the lv::BinClassifMetrics
formulas (modules/datasets/include/litiv/datasets/metrics.hpp:203-256), in numpy / plain Python, with
the reference's operation order for the metrics. Loaded only by tests/ as the checker.
"""
import math

import numpy as np

POSITIVE, NEGATIVE, OUTOFSCOPE, UNKNOWN, SHADOW = 255, 0, 85, 170, 50  # metrics.hpp:23-27


def accumulate(mask, gt, roi=None, counts=None):
    """counts = [TP, TN, FP, FN, SE, DC] (metrics.cpp:21-61)."""
    c = list(counts) if counts is not None else [0] * 6
    mask = np.asarray(mask, np.uint8)
    if gt is None:
        c[5] += mask.size
        return c
    gt = np.asarray(gt, np.uint8)
    care = (gt != OUTOFSCOPE) & (gt != UNKNOWN)
    if roi is not None:
        care &= np.asarray(roi, np.uint8) != NEGATIVE
    mp, gp = mask == POSITIVE, gt == POSITIVE
    c[0] += int((care & mp & gp).sum())
    c[1] += int((care & ~mp & ~gp).sum())
    c[2] += int((care & mp & ~gp).sum())
    c[3] += int((care & ~mp & gp).sum())
    c[4] += int((care & (gt == SHADOW) & mp).sum())
    c[5] += int((~care).sum())
    return c


def metrics(c):
    """[recall, specificity, FPR, FNR, PBC, precision, F-measure, MCC] (metrics.hpp:214-255)."""
    TP, TN, FP, FN = c[0], c[1], c[2], c[3]
    recall = TP / (TP + FN) if (TP + FN) > 0 else 0.0
    precision = TP / (TP + FP) if (TP + FP) > 0 else 0.0
    spec = TN / (TN + FP) if (TN + FP) > 0 else 0.0
    fpr = FP / (FP + TN) if (FP + TN) > 0 else 0.0
    fnr = FN / (TP + FN) if (TP + FN) > 0 else 0.0
    total = TP + TN + FP + FN
    pbc = 100.0 * (FN + FP) / total if total > 0 else 0.0
    fm = 2.0 * (recall * precision) / (recall + precision) if (recall + precision) > 0 else 0.0
    if (TP + FP) > 0 and (TP + FN) > 0 and (TN + FP) > 0 and (TN + FN) > 0:
        mcc = ((float(TP) * TN) - float(FP * FN)) / math.sqrt((float(TP) + FP) * float(TP + FN) * float(TN + FP) * float(TN + FN))
    else:
        mcc = 0.0
    return [recall, spec, fpr, fnr, pbc, precision, fm, mcc]
