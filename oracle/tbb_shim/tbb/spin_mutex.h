// Stand-in for TBB's spin_mutex: the reference only names the type
// (src/lgca_bitset.h:25,36); nothing locks it.  Oracle build only.
#pragma once
namespace tbb { struct spin_mutex { struct scoped_lock { explicit scoped_lock(spin_mutex &) {} }; }; }
