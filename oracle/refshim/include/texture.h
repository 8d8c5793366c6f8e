/* Empty stand-in: the harness uses no textures.  Test infrastructure. */
#pragma once
