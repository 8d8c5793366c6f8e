/* Empty stand-in: the harness uses no graphics interop.  Test infrastructure. */
#pragma once
