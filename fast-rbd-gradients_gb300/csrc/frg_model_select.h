// The robot compiled into this build: the tables header FRG_MODEL_TABLES names
// (written by frg/urdf.py from a URDF), else the iiwa_14 of utils/iiwa_14.urdf,
// the reference's only model.
#pragma once
#ifdef FRG_MODEL_TABLES
#include FRG_MODEL_TABLES
#else
#include "frg_model_iiwa14.h"
#endif
