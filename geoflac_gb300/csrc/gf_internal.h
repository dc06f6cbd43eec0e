// Host helpers shared between translation units of the library (not ABI).
#pragma once
#include "../../include/geoflac_gb300.h"

int gf_host_geotherm_columns(gf_params *p, gf_layout *L, int zone, int i_first, int i_last);
void gf_host_mesh_template(int n, int nzon, const int *nelz, const double *sizez, double *t, double *all_ratio);
int gf_host_restart_bc(gf_params *p, gf_layout *L);
