// TDVP engine (work in progress): entry points return "not implemented".
#include "common.cuh"
using namespace qca;
extern "C" {
#define NI(name, ...) int name(__VA_ARGS__) { set_error(#name ": not implemented"); return QCA_ERR_INVALID; }
NI(qca_engine_create, int, size_t, qca_engine**)
NI(qca_engine_destroy, qca_engine*)
NI(qca_chain_footprint, const qca_chain_desc*, int, size_t*)
NI(qca_chain_add, qca_engine*, const qca_chain_desc*, void*, int*)
NI(qca_chain_remove, qca_engine*, int)
NI(qca_engine_step, qca_engine*, int, void*)
NI(qca_engine_step_chains, qca_engine*, const int*, int, int, void*)
NI(qca_chain_measure, qca_engine*, int, double*, double*, double*, double*, void*)
NI(qca_chain_bonds, qca_engine*, int, int*)
NI(qca_chain_get_mps, qca_engine*, int, double*, size_t, void*)
NI(qca_chain_stats, qca_engine*, int, double*)
}
