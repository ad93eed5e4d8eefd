// Stand-in for spglib: the harness never calls it.
#pragma once
struct SpglibDataset;
extern "C" void spg_free_dataset(SpglibDataset*);
