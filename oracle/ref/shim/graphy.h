/* Host-only build of the reference: the X11/GL viewer is out of scope and absent, its
 * entry points do nothing. */
#pragma once
template <class... A> inline void graphy_render_points(A...) {}
template <class... A> inline void graphy_render_points3f(A...) {}
template <class... A> inline void graphy_render_points_size(A...) {}
template <class... A> inline void graphy_render_pointsEx(A...) {}
template <class... A> inline void graphy_render_points3(A...) {}
template <class... A> inline void graphy_set_3d(A...) {}
template <class... A> inline void graphy_set_orthographic(A...) {}
template <class... A> inline void graphy_close_display(A...) {}
template <class... A> inline void graphy_display_pixels(A...) {}
template <class... A> inline void graphy_render_lines(A...) {}
