// d2f_solver.h — the solver handle shared by the C ABI translation units.
#pragma once
#include "../../include/d2f.h"

struct d2f_solver {
    d2f_scene_desc d;
    int grid;  // launched blocks (cs > 1: clusters x cs)
    int smem;
    int cs;    // blocks per scene (one cluster)
};

extern thread_local char g_err[512];
int d2f_fail(int code, const char *msg);
int d2f_default_threads(const d2f_scene_desc &d);
