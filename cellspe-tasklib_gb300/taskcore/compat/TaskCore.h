// Stand-in for the swspectrometer's computing-core interface
// (spectrometer/src/TaskCore.h:36-89), used where that source tree is not on
// the include path.  The virtual methods are declared in the original's
// order, so a core built against either header has the same vtable layout.
#ifndef TASKCORE_H
#define TASKCORE_H

#include "Settings.h"

class Buffer;

class TaskCore
{
public:
   TaskCore(int) {}
   TaskCore() {}
   virtual ~TaskCore() {}

   // one-time set-up from the global settings
   virtual void prepare(swspect_settings_t* settings) = 0;
   // start work on the raw buffers (asynchronous); 0 when started
   virtual int run(Buffer** inbuf, Buffer** outbuf, Buffer** xpolbuf, Buffer** pcalbuf) = 0;
   // wait; number of complete spectra in the output buffers, or -1
   virtual int join() { return 1; }
   // release everything; 0 on success
   virtual int finalize() { return 0; }
   // add this core's spectra (auto, then cross) and phase-cal into the buffers
   virtual int combineResults(Buffer** outbuf, Buffer** pcalbuf) { return 0; }
   // set a buffer to 0.0 floats
   virtual void resetBuffer(Buffer* buf) {}
};

#endif // TASKCORE_H
