// ORACLE — test infrastructure only (see oracle_common.hpp).
//
// src/scheme_mhd_v2.hpp names bsp::tree_index_t<3>, which the reference does
// not define (the block index type it means is mesh::block_index_t). This
// alias, force-included by oracle/Makefile where it compiles the reference,
// lets scheme_mhd_v2.cpp compile unmodified from the reference checkout.
#pragma once
#include "mesh_block_index.hpp"

namespace bsp {
template<unsigned long Rank>
using tree_index_t = mesh::block_index_t<Rank>;
}
