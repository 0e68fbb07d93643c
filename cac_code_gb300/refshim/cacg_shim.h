// Reference-side plug-ins for libcacg: the state a GPU style needs, carried
// from the reference's own objects into one libcacg handle per CAC instance.
//
// The reference (fangyuanxiao/CAC_Code) keeps its state in host arrays owned
// by Atom (x, v, f, atom.h:40), Element (nodex, nodev, nodef, element.h:25)
// and Domain (boxlo, boxhi, periodicity, domain.h:17-40); memory->create lays
// them out contiguously (memory.h:115-260), so each crosses the C ABI as one
// pointer.  A GPU style forwards its virtuals to the ABI and maps a nonzero
// status to error->all, the reference's only error path.
//
// Build: compile these files with the reference sources (-I<reference>
// -I<repo>/include) and link libcacg.so; register the styles through the
// PairStyle / FixStyle lines of their headers (style_pair.h, style_fix.h)
// and construct NeighborGPU in place of Neighbor (cac.cpp:161).
#ifndef CACG_SHIM_H
#define CACG_SHIM_H

#include "cacg.h"
#include "pointers.h"

namespace CAC_NS {

class CacgShim : protected Pointers {
 public:
  // the instance's shim, created on first use
  static CacgShim *of(class CAC *cac);
  static void release(class CAC *cac);

  cacg_handle h;
  int tables_pending;  // a pair style's tables changed since they were handed over
  int ready;           // cacg_init and cacg_setup done on the current state

  // a nonzero status from the ABI becomes error->all with the library's message
  void check(int rc);
  // box, units, masses, atoms, element types, elements, neighbor settings and
  // the pair_style line into the handle (Pair::init_style time)
  void begin(const char *pair_style_line);
  // the atom and node positions and velocities of the host arrays into the handle
  void put_state();
  // x, v (atoms) and nodex, nodev (elements) back into the host arrays
  void get_state();
  // tables handed over: cacg_init, then cacg_setup from the current state
  void finish_init();

 private:
  explicit CacgShim(class CAC *cac);
  ~CacgShim();
};

}  // namespace CAC_NS

#endif
