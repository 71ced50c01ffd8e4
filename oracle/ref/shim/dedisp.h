/* Type stand-ins for the dedisp header the reference includes; the dedisp
 * library itself is not part of the reference and is not emulated. */
#pragma once
typedef struct dedisp_plan_struct *dedisp_plan;
typedef unsigned long dedisp_size;
typedef float dedisp_float;
typedef unsigned char dedisp_byte;
typedef int dedisp_bool;
typedef int dedisp_error;
