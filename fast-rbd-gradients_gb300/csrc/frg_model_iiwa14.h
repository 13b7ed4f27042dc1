/* Model tables of iiwa_14: written by frg/urdf.py from utils/iiwa_14.urdf.
 * Per joint k: F = R^T of the joint frame in its parent's frame (column-major
 * 3x3, the joint turning about z), the joint origin r in the parent frame, and
 * the link inertial (Ixx Ixy Ixz Iyy Iyz Izz at the COM, COM x y z, mass) in
 * the link frame.  FRG_MODEL_DQ_COLUMN0_ZERO is 1 when gravity (-z of the
 * base) lies along the first joint's axis, which makes column 0 of d tau / dq
 * vanish identically. */
#pragma once
#define FRG_MODEL_NAME "iiwa_14"
#define FRG_MODEL_NUM_JOINTS 7
#define FRG_MODEL_DQ_COLUMN0_ZERO 1
#define FRG_MODEL_JOINT_F { \
    {1.0, 0.0, 0.0, 0.0, 1.0, 0.0, 0.0, 0.0, 1.0}, \
    {-1.0, 0.0, 0.0, 0.0, 0.0, 1.0, 0.0, 1.0, 0.0}, \
    {-1.0, 0.0, 0.0, 0.0, 0.0, 1.0, 0.0, 1.0, 0.0}, \
    {1.0, 0.0, 0.0, 0.0, 0.0, -1.0, 0.0, 1.0, 0.0}, \
    {-1.0, 0.0, 0.0, 0.0, 0.0, 1.0, 0.0, 1.0, 0.0}, \
    {1.0, 0.0, 0.0, 0.0, 0.0, -1.0, 0.0, 1.0, 0.0}, \
    {-1.0, 0.0, 0.0, 0.0, 0.0, 1.0, 0.0, 1.0, 0.0}, }
#define FRG_MODEL_JOINT_ORIGIN { \
    {0.0, 0.0, 0.1575}, \
    {0.0, 0.0, 0.2025}, \
    {0.0, 0.2045, 0.0}, \
    {0.0, 0.0, 0.2155}, \
    {0.0, 0.1845, 0.0}, \
    {0.0, 0.0, 0.2155}, \
    {0.0, 0.081, 0.0}, }
#define FRG_MODEL_LINK_INERTIAL { \
    {0.121, 0.0, 0.0, 0.116, -0.021, 0.0175, 0.0, -0.03, 0.12, 5.76}, \
    {0.0638, 0.0001, 8e-05, 0.0416, 0.0157, 0.0331, 0.0003, 0.059, 0.042, 6.35}, \
    {0.0873, 0.0, 0.0, 0.083, 0.014, 0.0108, 0.0, 0.03, 0.13, 3.5}, \
    {0.0368, 0.0, 0.0, 0.02045, 0.008, 0.02171, 0.0, 0.067, 0.034, 3.5}, \
    {0.0318, 7e-06, 2.7e-05, 0.028916, 0.005586, 0.006, 0.0001, 0.021, 0.076, 3.5}, \
    {0.0049, 0.0, 0.0, 0.0047, 0.0, 0.0036, 0.0, 0.0006, 0.0004, 1.8}, \
    {0.0055, 0.0, 0.0, 0.0055, 0.0, 0.005, 0.0, 0.0, 0.02, 1.2}, }
