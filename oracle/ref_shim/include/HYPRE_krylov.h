/* Stub: see HYPRE.h in this directory. */
#pragma once
#include "HYPRE.h"
