/* Stand-in for the reference's OpenGL drawable base class: the fixed-body
 * classes derive from it, the harness never draws.  Test infrastructure. */
#pragma once
class Drawable {
public:
    virtual ~Drawable() {}
};
