/* world.h -- host-side construction of the seed-independent world description.
 *
 * Reads the data root layout of the reference engine (data/climate-<V>.txt, data/params/<V>/*.tsv;
 * engine/mc_data.h:84-183), builds the NormalNoise specifications (engine/mc_noise.h:178-252), the
 * offset spline, and the biome R-tree (engine/mc_biomes.h:128-212), and flattens the tree for the
 * device (children of a node contiguous, traversal order preserved).
 */
#ifndef MG_WORLD_H
#define MG_WORLD_H
#include <string>
#include <vector>

#include "mg_types.h"

namespace mg {

int version_from_name(const char *s);          /* "26.1".."26.4-snapshot-2" -> MG_V26_x, or -1 */
const char *version_name(int v);
int biome_count();
const char *biome_key(int id);                 /* "plains" (no namespace) */
int biome_from_key(const char *name);          /* accepts "minecraft:" prefix; -1 if unknown */

/* Presets per dimension in mcgen_preset_name order. */
int preset_count(int dim);
const char *preset_name(int dim, int i);

/* Build the description of (version, dim, preset).  Returns 0 or an MCGEN_E_* code with err set. */
int build_world(const char *root, int version, int dim, const char *preset, MgWorldDesc *desc,
                std::vector<MgTreeNode> *tree, std::string *err);

/* BiomeManager.obfuscateSeed: first 8 bytes of SHA-256 of the little-endian seed. */
int64_t obfuscate_seed(int64_t seed);

}  // namespace mg
#endif
