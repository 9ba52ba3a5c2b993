/*
 * Stand-in "rebound.h" used ONLY to compile the unmodified ASSIST sources into
 * the checker library oracle/_ref/libassist_ref.so.  It reuses the REBOUND
 * subset declared by this project (include/rebound.h) and adds the few
 * declarations ASSIST's assist.c / tools.c reference at compile time but never
 * reach on the force path (archive interpolation, particle merging).
 */
#ifndef ORACLE_REF_STANDIN_REBOUND_H
#define ORACLE_REF_STANDIN_REBOUND_H
#include "../../include/rebound.h"
#ifdef __cplusplus
extern "C" {
#endif
void reb_simulation_create_from_simulationarchive_with_messages(struct reb_simulation* r,
        struct reb_simulationarchive* sa, long snapshot, enum reb_simulation_binary_error_codes* warnings);
struct reb_particle reb_particle_com_of_pair(struct reb_particle p1, struct reb_particle p2);
#ifdef __cplusplus
}
#endif
#endif
