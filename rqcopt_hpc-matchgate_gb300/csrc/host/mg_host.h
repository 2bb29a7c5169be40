/*
 * Definitions shared by the host-layer files (csrc/host): GPU target handles and the
 * brickwall-to-sequential-circuit expansion.
 */
#pragma once

#include "matchgate.h"
#include "../mg_internal.h"

#define MG_TARGET_MAGIC 0x6d677467u

/* what mg_target_* returns: a tagged handle of a GPU target */
typedef struct
{
	unsigned magic;
	int L;
	mgcu_target* dev;
} mg_target_handle;

/* brickwall -> sequential circuit with one block per layer (src/matchgate_target.c:308-324) */
typedef struct { struct matchgate* gates; int* wires; int* block; int ngates; } seq_circuit;
int brickwall_seq(const struct matchgate vlist[], int nlayers, int L, const int* perms[], seq_circuit* s);
void seq_free(seq_circuit* s);
