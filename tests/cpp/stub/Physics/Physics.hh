// stand-in: see spheral_stub.hh
#include "../spheral_stub.hh"
