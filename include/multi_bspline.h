/*
 * multi_bspline.h -- umbrella header (replaces src/multi_bspline.h): the
 * uniform 3D multi-spline create/set/eval API of einspline, GPU-resident.
 */
#ifndef EINSPLINE_GB300_MULTI_BSPLINE_H
#define EINSPLINE_GB300_MULTI_BSPLINE_H

#include "bspline_base.h"
#include "multi_bspline_structs.h"
#include "multi_bspline_create.h"
#include "multi_bspline_eval_s.h"
#include "multi_bspline_eval_d.h"
#include "multi_bspline_eval_c.h"
#include "multi_bspline_eval_z.h"

#endif
